"""CPU checks of index plans and recurrences that kernels rely on (no GPU).

* The tensor-copy plane gather of the multi-pass filter kernel (csrc/k_dsm.cu,
  k_dsm_b<float, true>): a 40 x 10 box of the canonical arrays starting 4
  columns before the tile's halo column and one row before the tile, with the
  periodic halo columns written afterwards, supplies every value an owned
  point reads with a nonzero filter weight exactly as the per-element gather
  does (periodic in x, rows clamped to the interior), for tiles at both seams
  and grids whose nxp is a multiple of 32 or of 4 only.
* The seam band of the one-pass dynamic Smagorinsky kernel (seam_row and
  seam_line in csrc/cf_internal.cuh, enumerated by k_dsm_seam in
  csrc/k_dsm_fused.cu): every centre whose stencil reaches a wall ghost entry
  that is not a periodic copy lies in the band, and the enumeration covers the
  band exactly once.
* The continuant form of the eqwm elimination (csrc/k_eqwm.cu, split path):
  as accurate as the reference's Thomas sweep against exact rational
  elimination of the same coefficients (eqwm.f90:52-88, 121-205).
"""
import itertools
import math
import os
import random
import re
from fractions import Fraction

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "channel-flow_gb300", "csrc")


def _const(path, name):
    text = open(os.path.join(CSRC, path)).read()
    m = re.search(r"\b" + name + r"\s*=\s*([^,;]+)[,;]", text)
    assert m, name
    return m.group(1).strip()


def test_tensor_copy_box_plus_halo_columns_reproduce_the_gather():
    dbx = int(_const("k_dsm.cu", "DB_X"))
    dby = int(_const("k_dsm.cu", "DB_Y"))
    assert (dbx, dby) == (32, 8)
    bx_w, by_h, ox = dbx + 8, dby + 2, 3  # DBT_BX, DBT_BY, DBT_OX
    assert _const("k_dsm.cu", "DBT_BX") == "DB_X + 8" and _const("k_dsm.cu", "DBT_OX") == "3"

    def check(nxp, nym):
        val = lambda x, y: (x + 1) * 1000 + (y + 1)
        nyg = nym + 2
        for bx, by in itertools.product(range(-(-nxp // dbx)), range(-(-nym // dby))):
            x0, y0 = bx * dbx - 4, by * dby - 1
            assert (x0 * 4) % 16 == 0  # the TMA x coordinate rule for 4-byte elements
            box = [[val(x0 + c, y0 + r) if 0 <= x0 + c < nxp and 0 <= y0 + r < nym else 0
                    for c in range(bx_w)] for r in range(by_h)]
            sxr = nxp - bx * dbx + 1
            for side, col, src in ((0, 0, nxp - 1), (1, sxr, 0)):
                if (side == 0 and bx == 0) or (side == 1 and 1 <= sxr <= dbx + 1):
                    for sy in range(by_h):
                        y = by * dby - 1 + sy
                        if 0 <= y < nym:
                            box[sy][ox + col] = val(src, y)
            i0, j0 = 2 + bx * dbx, 2 + by * dby
            for tx, ty in itertools.product(range(dbx), range(dby)):
                i, j = i0 + tx, j0 + ty
                if i > nxp + 1 or j > nyg - 1:
                    continue
                for d in (-1, 0, 1):
                    for dy, live in ((-1, j != 2), (0, True), (1, j != nyg - 1)):
                        if not live:
                            continue
                        ii = i + d
                        ii = ii + nxp if ii < 2 else (ii - nxp if ii > nxp + 1 else ii)
                        jj = min(max(j + dy, 2), nyg - 1)
                        assert box[ty + 1 + dy][tx + 1 + d + ox] == val(ii - 2, jj - 2), (nxp, nym, bx, by, tx, ty)

    for nxp in (40, 44, 48, 64, 100, 192, 256):
        for nym in (10, 15, 64):
            check(nxp, nym)


def _seam_row(j, nyg):
    return j <= 3 or j >= nyg - 2


def _seam_line(i, n):
    return i <= 3 or i >= n


def test_seam_band_holds_every_centre_that_reads_a_nonperiodic_wall_ghost():
    """Dependencies of a centre's L.M, M.M and |S| on the raw fields, as the
    multi-pass route forms them: the stage-A quantities of the 27 neighbours
    (compute_Sij reads U at x faces i-1..i, rows j-1..j+1, planes k-1..k+1 and
    W at centres i-1..i+1, rows j-1..j+1, faces k-1..k; a ghost neighbour
    takes its canonical twin's) and every filtered-velocity element around the
    centre (a 27-point filter of the field around the element, a ghost element
    its twin's) -- more than compute_Sij of Uf reads.  Every wall ghost row
    entry of U and W outside the canonical columns and planes is taken as
    possibly not a periodic copy (the equilibrium wall model's Neumann values
    use alpha at the ghost's own position; compared with the oracle, U's
    differ at column 1, column nx and planes 1, nzg-1, nzg, W's at column 1
    and plane 1)."""
    nxp, nzp, nyg = 12, 10, 14
    nx, nzg, nz, nxg = nxp + 2, nzp + 3, nzp + 2, nxp + 3
    wrap = lambda i, n: 2 + (i - 2) % n
    canon = lambda i, k: 2 <= i <= nxp + 1 and 2 <= k <= nzp + 1
    bad_u = {(i, j, k) for j in (1, nyg) for i in range(1, nx + 1) for k in range(1, nzg + 1) if not canon(i, k)}
    bad_w = {(i, j, k) for j in (1, nyg) for i in range(1, nxg + 1) for k in range(1, nz + 1) if not canon(i, k)}

    def q_reads(i, j, k):  # stage-A quantities at a canonical centre
        i, k = wrap(i, nxp), wrap(k, nzp)
        u = {(a, b, c) for a in (i - 1, i) for b in (j - 1, j, j + 1) for c in (k - 1, k, k + 1)}
        w = {(a, b, c) for a in (i - 1, i, i + 1) for b in (j - 1, j, j + 1) for c in (k - 1, k)}
        return u, w

    def f_reads(i, j, k):  # a filtered-velocity element (U or W grid), canonical twin
        i, k = wrap(i, nxp), wrap(k, nzp)
        return {(a, b, c) for a in (i - 1, i, i + 1) for b in (j - 1, j, j + 1) for c in (k - 1, k, k + 1)}

    for i in range(2, nxp + 2):
        for k in range(2, nzp + 2):
            for j in range(2, nyg):
                ru, rw = set(), set()
                for di, dj, dk in itertools.product((-1, 0, 1), repeat=3):
                    if 2 <= j + dj <= nyg - 1:
                        u, w = q_reads(i + di, j + dj, k + dk)
                        ru |= u
                        rw |= w
                for di, dj, dk in itertools.product((-1, 0, 1), repeat=3):
                    ru |= f_reads(i + di, j + dj, k + dk)
                    rw |= f_reads(i + di, j + dj, k + dk)
                if (ru & bad_u) or (rw & bad_w):
                    assert _seam_row(j, nyg) and (_seam_line(i, nxp) or _seam_line(k, nzp)), (i, j, k)

    # the enumeration of k_dsm_seam: band columns (every plane), then band
    # planes at the columns 4..nxp-1
    for np_x, np_z in ((12, 10), (16, 16), (7, 9), (5, 6), (4, 4), (3, 5)):
        band = lambda n: sorted({c for c in (2, 3, n, n + 1) if 2 <= c <= n + 1})
        xs, zs, nxr = band(np_x), band(np_z), max(0, np_x - 4)
        pts = [(x, k) for x in xs for k in range(2, np_z + 2)] + [(4 + q % nxr, zs[q // nxr])
                                                                  for q in range(len(zs) * nxr)]
        want = [(i, k) for i in range(2, np_x + 2) for k in range(2, np_z + 2)
                if _seam_line(i, np_x) or _seam_line(k, np_z)]
        assert sorted(pts) == sorted(want) and len(pts) == len(set(pts)), (np_x, np_z)


def _grid(ncv, h, s):
    d = [s ** i for i in range(ncv)]
    tot = sum(d)
    yfa = [0.0]
    for q in range(ncv):
        yfa.append(yfa[-1] + h * d[q] / tot)
    return [None] + [0.5 * (yfa[q] + yfa[q + 1]) for q in range(ncv)], [None] + yfa


def _coefficients(tau, nu, ncv, ycv, yfa):
    idcv = [0.0] * (ncv + 1)
    for q in range(1, ncv):
        idcv[q] = 1.0 / (ycv[q + 1] - ycv[q])
    rw = 1.0 / (ycv[1] - yfa[1])
    ut = math.sqrt(tau)
    c1, cd = 0.41 * ut, ut / nu / 17.0
    mu = [0.0] * (ncv + 1)
    for q in range(ncv, 1, -1):
        dd = 1.0 - math.exp(-(yfa[q] * cd))
        mu[q] = nu + c1 * yfa[q] * dd * dd
    return idcv, rw, mu


def _thomas(u, nu, ncv, idcv, rw, mu):
    al, be = u, 0.0
    for q in range(ncv - 1, 1, -1):
        sup, sub = mu[q + 1] * idcv[q], mu[q] * idcv[q - 1]
        m = -(sup + sub) + sup * be
        al, be = -sup * al / m, -sub / m
    sup = mu[2] * idcv[1]
    return nu * (-sup * al / (-(sup + nu * rw) + sup * be)) * rw


def _continuant(u, nu, ncv, idcv, rw, mu):
    dn1, dn2, a, subp = 1.0, 0.0, u, 0.0
    sup = mu[ncv] * idcv[ncv - 1]
    for q in range(ncv - 1, 1, -1):
        sub = mu[q] * idcv[q - 1]
        dn = -(sup + sub) * dn1 - (sup * subp) * dn2
        a, dn2, dn1, subp, sup = -sup * a, dn1, dn, sub, sub
        if q % 8 == 0:
            e = math.frexp(dn1)[1]
            if abs(e) > 512:
                sc = 2.0 ** (-e)
                dn1, dn2, a = dn1 * sc, dn2 * sc, a * sc
    return nu * (-sup * a / (-(sup + nu * rw) * dn1 - sup * subp * dn2)) * rw


def _exact(u, nu, ncv, idcv, rw, mu):
    F = Fraction
    al, be = F(u), F(0)
    for q in range(ncv - 1, 1, -1):
        sup, sub = F(mu[q + 1]) * F(idcv[q]), F(mu[q]) * F(idcv[q - 1])
        m = -(sup + sub) + sup * be
        al, be = -sup * al / m, -sub / m
    sup = F(mu[2]) * F(idcv[1])
    return float(F(nu) * (-sup * al / (-(sup + F(nu) * F(rw)) + sup * be)) * F(rw))


@pytest.mark.parametrize("ncv", [3, 30, 45])
def test_continuant_elimination_as_accurate_as_thomas(ncv):
    rng = random.Random(ncv)
    worst_c = worst_t = 0.0
    for _ in range(25):
        retau = math.exp(rng.uniform(math.log(300), math.log(20000)))
        nu = 2.0 / (retau / 0.09) ** (1 / 0.88)
        h = rng.uniform(0.03, 0.3)
        ut = retau * nu
        u = ut * (math.log(h * ut / nu) / 0.41 + 5.2) * rng.uniform(0.6, 1.4)
        ycv, yfa = _grid(ncv, h, 1.10)
        idcv, rw, mu = _coefficients(ut * ut * rng.uniform(0.5, 2.0), nu, ncv, ycv, yfa)
        x = _exact(u, nu, ncv, idcv, rw, mu)
        worst_c = max(worst_c, abs(_continuant(u, nu, ncv, idcv, rw, mu) - x) / abs(x))
        worst_t = max(worst_t, abs(_thomas(u, nu, ncv, idcv, rw, mu) - x) / abs(x))
    assert worst_c < 1e-13 and worst_c < 4 * max(worst_t, 1e-16), (worst_c, worst_t)
