"""The learned wall-stress model: the batched eqwm labeller against the
oracle's solve_u_eqwm (eqwm.f90:90-223), the network's forward pass and
gradient against the numpy restatement (oracle/mlp_oracle.py), training to
the 2 % target and what the trained network gains over the eqwm solve."""
import math

import numpy as np
import pytest

from conftest import ROOT


def _oracle_mlp():
    import sys, os
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mlp_oracle
    return mlp_oracle


def test_oracle_gradient_matches_finite_differences(monkeypatch):
    """The numpy backward pass against central differences of its forward
    pass, with the BF16 rounding switched off so that the loss is smooth."""
    mo = _oracle_mlp()
    monkeypatch.setattr(mo, "bf16", lambda a: np.asarray(a, dtype=np.float32))
    rng = np.random.default_rng(0)
    p = (rng.standard_normal(mo.NPARAM) * 0.3).astype(np.float32)
    x = rng.standard_normal((64, 3)).astype(np.float32)
    t = rng.standard_normal(64).astype(np.float32)
    g, _ = mo.gradient(p, x, t)
    loss = lambda q: float(np.mean((mo.forward(q, x)["y"].astype(np.float64) - t) ** 2))
    idx = np.r_[rng.choice(np.arange(0, 192), 6), rng.choice(np.arange(256, 4352), 12), [4352, 4420, 4480]]
    for i in idx:
        e = 1e-2
        qp, qm = p.copy(), p.copy()
        qp[i] += e
        qm[i] -= e
        fd = (loss(qp) - loss(qm)) / (2 * e)
        assert abs(fd - g[i]) <= 2e-2 * max(abs(g).max() * 0.05, abs(g[i])), (i, fd, g[i])


@pytest.mark.gpu
def test_eqwm_batch_matches_oracle():
    import torch
    import sys, os
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from channelflow import wallmlp
    u, h, nu = wallmlp.training_inputs(200, seed=3)
    dev = torch.device("cuda:0")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    tau, it = wallmlp.eqwm_solve_batch(T(u), T(h), T(nu), ncv=30, stretch=1.10, tau_init=1e-3, iters=True)
    tau, it = tau.cpu().numpy(), it.cpu().numpy()
    same = 0
    for q in range(200):
        to, io = oracle.solve_u_eqwm(u[q], nu[q], h[q], 30, 1.10, 1e-3)
        assert abs(tau[q] - to) <= 1e-9 * abs(to), (q, tau[q], to)
        same += int(io == it[q])
    assert same >= 196  # the stopping test may flip at its threshold
    assert (it < 100).all()


def _data(n, seed, dev, operating=False):
    """Training samples, or (operating=True) samples of the operating range."""
    from channelflow import wallmlp
    kw = wallmlp.OPERATING if operating else {}
    return wallmlp.training_set(n, seed=seed, device=dev, ncv=30, stretch=1.10, **kw)


@pytest.mark.gpu
def test_forward_and_gradient_match_oracle():
    import torch
    from channelflow import wallmlp
    mo = _oracle_mlp()
    dev = torch.device("cuda:0")
    u, h, nu, tau = (a[:896] for a in _data(1024, 5, dev))  # a multiple of 128
    net = wallmlp.WallMLP(seed=1)
    net.fit_normalisation(u, h, nu, tau)
    p, norm, env = net.get()
    un, hn, nn_, tn = (a.cpu().numpy() for a in (u, h, nu, tau))
    # normalisation: means / deviations of the FP32 logs and of the target
    lu, lh, ln = (np.log(a.astype(np.float32)) for a in (un, hn, nn_))
    logs = [a.astype(np.float64) for a in (lu, lh, ln, np.log(tn.astype(np.float32)) - (ln + lu - lh))]
    for c in range(4):
        assert abs(norm[c] - logs[c].mean()) <= 1e-6 * max(1.0, abs(norm[c]))  # logf vs numpy: an ulp
        assert abs(norm[4 + c] - logs[c].std()) <= 1e-6 * norm[4 + c]
    # forward on the FP32 pipes
    got = net.predict(u, h, nu, tensor_cores=False).cpu().numpy()
    want = mo.predict_tau(p, norm, un, hn, nn_)
    d = np.abs(got / want - 1)
    # an ulp of difference before a BF16 rounding can flip one activation
    assert np.median(d) < 1e-6 and np.mean(d > 1e-5) < 0.02 and d.max() < 2e-3, (np.median(d), d.max())
    # gradient over the batch: layer 2 on the tensor cores (BF16 output
    # gradient in its products), and on the FP32 pipes
    x = mo.features(un, hn, nn_, norm)
    t = mo.target(un, hn, nn_, tn, norm)
    for tc in (True, False):
        net.train_tensor_cores(tc)
        g, loss = net.gradient(u, h, nu, tau)
        go, lo = mo.gradient(p, x, t, delta_bf16=tc)
        g = g.cpu().numpy()
        assert abs(loss - lo) <= 1e-4 * lo, (tc, loss, lo)
        err = np.max(np.abs(g - go)) / np.max(np.abs(go))
        print("tensor cores" if tc else "FP32 pipes", "gradient error", err)
        assert err <= 1e-4, (tc, err)
        # layer 2's weight gradient on its own (the tensor-core product)
        gw, gwo = g[mo.O_W2:mo.O_B2], go[mo.O_W2:mo.O_B2]
        assert np.max(np.abs(gw - gwo)) <= 1e-4 * np.max(np.abs(gwo)), tc
    net.train_tensor_cores(True)


@pytest.mark.gpu
def test_training_reaches_two_percent_and_tensor_cores_match():
    """Trained on 2^18 eqwm samples; on held-out samples of the operating range
    the tensor-core inference stays within 2 % of eqwm (the untrained network
    does not), and agrees with the FP32-pipe inference."""
    import torch
    from channelflow import wallmlp
    dev = torch.device("cuda:0")
    u, h, nu, tau = _data(1 << 18, 11, dev)
    net = wallmlp.WallMLP(seed=2)
    net.fit_normalisation(u, h, nu, tau)
    ut, ht, nt, tt = _data(1 << 15, 12, dev, operating=True)
    before = (net.predict(ut, ht, nt) / tt - 1).abs().max().item()
    loss = net.train(u, h, nu, tau, epochs=30, batch=512, lr=3e-3, seed=0)
    print("loss", loss[0], loss[-1])
    assert loss[-1] < loss[0] * 1e-2, loss
    tc, inside = net.predict(ut, ht, nt, tensor_cores=True, inside=True)
    cc = net.predict(ut, ht, nt, tensor_cores=False)
    m = inside.bool()
    assert m.float().mean().item() == 1.0  # the operating range lies inside the envelope
    err = (tc[m] / tt[m] - 1).abs()
    print("max", err.max().item(), "p99", err.quantile(0.99).item(), "mean", err.mean().item(), "before", before)
    d = ((tc - cc).abs() / cc)
    assert d.median().item() < 1e-6 and (d > 1e-5).float().mean().item() < 0.02 and d.max().item() < 2e-3
    assert err.max().item() < 0.02 and before > 0.5


@pytest.mark.gpu
def test_learned_stress_in_the_wall_model():
    """A trained network serving the wall stress of the equilibrium wall model
    (channel with eqwm, Re_tau 2000): ten fast-path steps stay close to the
    eqwm run, the checked error stays within 2 %, and points outside the
    envelope fall back to eqwm."""
    import torch
    import channelflow as cf
    from channelflow import wallmlp
    from conftest import channel_case, rel_err
    dev = torch.device("cuda:0")
    u, h, nu, tau = _data(1 << 17, 21, dev)
    net = wallmlp.WallMLP(seed=4, ncv=30, stretch=1.10)
    net.fit_normalisation(u, h, nu, tau)
    net.train(u, h, nu, tau, epochs=30, batch=512, lr=3e-3, seed=1)
    case = channel_case(34, 33, 34, stretch=0.0, wall=3, retau=2000.0, profile="plug", jref=3, ncv=30)
    out = {}
    for use in (False, True):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_FP64, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        if use:
            ch.set_wall_mlp(net, check_every=5)
        ch.set_fixed_dt(case["dt"])
        ch.time_step_rk3(10)
        out[use] = ch.download()
        if use:
            log = ch.wall_mlp_log()
        ch.close()
    print(log)
    assert log["calls"] == 10 and log["served"] > 0.9 * (34 * 35 * 2)
    assert log["max_rel_err"] < 0.02
    for n in ("U", "W"):  # the velocity follows the stress: within its 2 %
        assert rel_err(out[True][n], out[False][n]) < 2e-2


@pytest.mark.gpu
def test_network_throughput_over_eqwm():
    """What the network gains over the method it replaces: wall-stress
    evaluations per second of the tensor-core inference against the eqwm
    solve on the same 2^20 inputs (warm start at the network's answer, so the
    solve does its fewest passes), CUDA-event timed."""
    import torch
    from channelflow import wallmlp
    dev = torch.device("cuda:0")
    u, h, nu, tau = _data(1 << 20, 31, dev)
    net = wallmlp.WallMLP(seed=6)
    net.fit_normalisation(u, h, nu, tau)
    n = u.numel()

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    t_nn = timed(lambda: net.predict(u, h, nu, tensor_cores=True))
    t_cc = timed(lambda: net.predict(u, h, nu, tensor_cores=False))
    t_eq = timed(lambda: wallmlp.eqwm_solve_batch(u, h, nu, ncv=30, stretch=1.10, tau_init=float(tau.mean())), reps=2)
    print(f"n={n} network(tensor cores) {t_nn:.3f} ms  network(FP32 pipes) {t_cc:.3f} ms  eqwm {t_eq:.3f} ms "
          f"-> {n / t_nn / 1e3:.3e} vs {n / t_eq / 1e3:.3e} evaluations/s, ratio {t_eq / t_nn:.1f}")
    assert t_eq / t_nn >= 5.0


@pytest.mark.gpu
def test_points_outside_the_envelope_fall_back_to_eqwm():
    """With an envelope that excludes every wall point the learned stress
    serves nothing: the run is bit-identical to the eqwm run and the record
    counts every point as a fallback."""
    import torch
    import channelflow as cf
    from channelflow import wallmlp
    from conftest import channel_case
    dev = torch.device("cuda:0")
    u, h, nu, tau = _data(1 << 12, 41, dev)
    net = wallmlp.WallMLP(seed=5, ncv=30, stretch=1.10)
    net.fit_normalisation(u, h, nu, tau)
    p, norm, env = net.get()
    env[:3] = env[3:] = -50.0  # an empty box far below every log input
    net.set(env=env)
    case = channel_case(18, 17, 18, stretch=0.0, wall=3, retau=2000.0, profile="plug", jref=3, ncv=30)
    out = {}
    for use in (False, True):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_FP64, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        if use:
            ch.set_wall_mlp(net, check_every=1)
        ch.set_fixed_dt(case["dt"])
        ch.time_step_rk3(3)
        out[use] = ch.download()
        if use:
            log = ch.wall_mlp_log()
        ch.close()
    assert log["calls"] == 3 and log["served"] == 0 and log["fallback"] == 18 * 19 * 2
    for n in ("U", "V", "W", "P", "nu_t"):
        assert np.array_equal(out[True][n], out[False][n]), n


@pytest.mark.gpu
def test_expired_tensor_core_wait_falls_back_to_eqwm():
    """With the test hook that makes the tensor-core inference issue no MMA,
    every bounded wait runs out: the kernel records it, frees its tensor
    memory and leaves all its samples to eqwm, so the step is bit-identical to
    the eqwm run; the record clears, and normal inference serves again."""
    import torch
    import channelflow as cf
    from channelflow import wallmlp
    from conftest import channel_case
    dev = torch.device("cuda:0")
    u, h, nu, tau = _data(1 << 15, 43, dev)
    net = wallmlp.WallMLP(seed=7, ncv=30, stretch=1.10)
    net.fit_normalisation(u, h, nu, tau)
    case = channel_case(18, 17, 18, stretch=0.0, wall=3, retau=2000.0, profile="plug", jref=3, ncv=30)
    out = {}
    for use in (False, True):
        ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_FP64, **case["prm"])
        ch.upload(case["U"], case["V"], case["W"])
        ch.init_mass_flow()
        ch.apply_boundary_conditions()
        if use:
            ch.set_wall_mlp(net, check_every=1)
            net.test_skip_mma(True)
        ch.set_fixed_dt(case["dt"])
        ch.time_step_rk3(1)
        out[use] = ch.download()
        if use:
            log = ch.wall_mlp_log()
            assert net.wait_expired()
            assert not net.wait_expired()  # the record was cleared
            net.test_skip_mma(False)
            ch.time_step_rk3(1)
            assert not net.wait_expired()
            assert ch.wall_mlp_log()["served"] > 0
        ch.close()
    assert log["calls"] == 1 and log["served"] == 0 and log["fallback"] == 18 * 19 * 2
    for n in ("U", "V", "W", "P", "nu_t"):
        assert np.array_equal(out[True][n], out[False][n]), n


@pytest.mark.gpu
def test_wall_model_inputs_are_the_solver_inputs():
    """cf_wall_model_inputs returns what the equilibrium wall model feeds to
    its eqwm solve: solving eqwm on those inputs (batched, cold start)
    reproduces the stress the wall-model call stored for every wall point."""
    import torch
    import channelflow as cf
    from channelflow import wallmlp
    from conftest import channel_case
    case = channel_case(34, 33, 34, stretch=0.0, wall=3, retau=2000.0, profile="plug", jref=3, ncv=30)
    ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_FP64, **case["prm"])
    ch.upload(case["U"], case["V"], case["W"])
    ch.apply_boundary_conditions()
    ch.compute_eddy_viscosity()
    ch.compute_wall_model()
    tau_wm = ch.download_wall()["tau_eqwm_initial"]
    u, h, nu = wallmlp.wall_model_inputs(ch)
    assert u.numel() == 34 * 2 * 35 and h == pytest.approx(case["y"][2] * 0.5 + case["y"][1] * 0.5, rel=1e-12)
    T = lambda v: torch.full_like(u, v)
    tau = wallmlp.eqwm_solve_batch(u, T(h), T(nu), ncv=30, stretch=1.10, tau_init=1e-3).cpu().numpy()
    want = np.ravel(tau_wm, order="F")
    assert np.abs(tau / want - 1).max() < 1e-5, np.abs(tau / want - 1).max()
    ch.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ncv", [30, 45, 60])
def test_split_eqwm_stress_matches_oracle_solve(ncv):
    """The split path's eqwm solve (FP32 Picard passes, then FP64 passes;
    for ncv <= 45 the later FP64 passes update the previous pass's
    exponentials by a Taylor factor instead of evaluating exp) against the
    oracle's solve_u_eqwm (eqwm.f90:90-223) of every wall point on the same
    inputs and warm start: both stop at the reference's criterion
    |d tau / tau_lam| < 1e-7, so they agree to a few 1e-7 of tau_lam."""
    from oracle import solve_u_eqwm
    import channelflow as cf
    from channelflow import wallmlp
    from conftest import channel_case
    case = channel_case(18, 17, 18, stretch=0.0, wall=3, retau=2000.0, profile="plug", jref=3, ncv=ncv)
    ch = cf.Channel(case["x"], case["y"], case["z"], precision=cf.PREC_SPLIT, **case["prm"])
    ch.upload(case["U"], case["V"], case["W"])
    ch.apply_boundary_conditions()
    ch.compute_eddy_viscosity()
    tau_in = np.ravel(ch.download_wall()["tau_eqwm_initial"], order="F")
    u, h, nu = wallmlp.wall_model_inputs(ch)
    u = u.cpu().numpy()
    ch.compute_wall_model()
    tau = np.ravel(ch.download_wall()["tau_eqwm_initial"], order="F")
    ch.close()
    ref = np.array([solve_u_eqwm(u[q], nu, h, ncv, 1.10, tau_in[q])[0] for q in range(u.size)])
    tau_lam = nu * u / h
    err = np.abs(tau - ref) / tau_lam
    assert np.all(np.isfinite(tau)) and err.max() < 2e-6, err.max()


@pytest.mark.gpu
def test_harvested_solver_samples():
    """Samples drawn from the solver's own wall-modelled runs across the
    operating range: finite, positive, labelled by eqwm, and mixed into a
    training set in the requested share."""
    import torch
    from channelflow import wallmlp
    dev = torch.device("cuda:0")
    runs = ((500.0, 4), (10000.0, 5))
    u, h, nu, steps = wallmlp.harvest_inputs(20000, device=dev, runs=runs, warm=50, every=10)
    assert u.numel() == 20000 and steps >= 2 * 60
    assert torch.isfinite(u).all() and (u > 0).all()
    assert len(torch.unique(h)) == 2 and len(torch.unique(nu)) == 2
    (tu, th, tn, tt), kept = wallmlp.training_set_mixed(1 << 14, solver_fraction=0.5, device=dev, seed=3)
    assert kept > 0.45 * (1 << 14) and tu.numel() > 0.9 * (1 << 14)
    assert torch.isfinite(tt).all() and (tt > 0).all()


@pytest.mark.gpu
def test_tensor_core_training_against_fp32_pipes():
    """The same two epochs trained with layer 2 on the tensor cores and on the
    FP32 pipes from the same start: both reduce the loss alike; the time per
    epoch of each is printed (CUDA events)."""
    import torch
    from channelflow import wallmlp
    dev = torch.device("cuda:0")
    u, h, nu, tau = _data(1 << 17, 51, dev)
    out = {}
    for tc in (True, False):
        net = wallmlp.WallMLP(seed=9)
        net.fit_normalisation(u, h, nu, tau)
        net.train_tensor_cores(tc)
        net.train(u, h, nu, tau, epochs=1, batch=4096, lr=3e-3, seed=0)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        loss = net.train(u, h, nu, tau, epochs=2, batch=4096, lr=3e-3, seed=1)
        e1.record()
        e1.synchronize()
        out[tc] = (loss, e0.elapsed_time(e1) / 2)
        net.close()
    print("ms per epoch of 2^17 samples, batch 4096: tensor cores %.3f, FP32 pipes %.3f" % (out[True][1], out[False][1]),
          "losses", out[True][0], out[False][0])
    for tc in (True, False):
        assert out[tc][0][-1] < out[tc][0][0]
    assert abs(out[True][0][-1] / out[False][0][-1] - 1) < 0.2
