// k_wmlp.cu -- learned wall-stress model: batched eqwm labelling, training
// and inference of a 3 -> 64 -> 64 -> 1 tanh network that stands in for the
// per-point ODE solve of the equilibrium wall model (solve_u_eqwm,
// eqwm.f90:90-223).  No counterpart in the reference.
//
// Parameters (FP32 master copy, 4481 values): W1[64][3], b1[64],
// W2[64][64] (row = output unit), b2[64], W3[64], b3.  The 64 x 64 layer --
// the tensor-core layer -- takes BF16 weights and BF16 inputs and
// accumulates in FP32; layers 1 and 3 run in FP32.  Training runs the three
// products of that layer (forward, input gradient, weight gradient) on the
// tensor cores with BF16 operands (the layer's output gradient rounded to
// BF16 where it feeds them), back-propagates through the rounding of the
// weights and inputs unchanged (straight-through) and updates the FP32
// master copy with Adam; an FP32-pipe gradient kernel is the cross-check.  Inputs are normalised logs,
// x = (log(u, h, nu) - mean)/std; the output is the normalised log of the
// stress over its laminar value, y = (log(tau h / (nu u)) - mean)/std, a
// bounded smooth function of the matching Reynolds number u h / nu.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "cf_internal.cuh"

namespace {

constexpr int MH = 64;  // hidden width
constexpr int O_W1 = 0, O_B1 = 192, O_W2 = 256, O_B2 = 4352, O_W3 = 4416, O_B3 = 4480, NP = 4481;
static_assert(NP == CF_MLP_NPARAM, "parameter count");

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// normalisation (float): means m[0..3] and reciprocal deviations r[0..3] of
// log u, log h, log nu and the target log(tau h/(nu u)); its standard
// deviation s3; envelope of the three input logs
struct MlpNorm {
    float m[4], r[4], s3;
    float lo[3], hi[3];
};

// returns log(nu u / h), the laminar stress's log, which the output is relative to
__device__ __forceinline__ float mlp_features(const MlpNorm &nm, double u, double h, double nu, float x[3], bool *in) {
    const float lu = logf((float)u), lh = logf((float)h), ln = logf((float)nu);
    x[0] = (lu - nm.m[0]) * nm.r[0];
    x[1] = (lh - nm.m[1]) * nm.r[1];
    x[2] = (ln - nm.m[2]) * nm.r[2];
    if (in) *in = lu >= nm.lo[0] && lu <= nm.hi[0] && lh >= nm.lo[1] && lh <= nm.hi[1] && ln >= nm.lo[2] && ln <= nm.hi[2];
    return ln + lu - lh;
}

// ---------------------------------------------------------------------------
// Batched eqwm (FP64): one thread per sample, the recurrence of the wall
// model kernel on the unit ODE grid scaled by the sample's matching height
// (eqwm.f90:20-50 scales the grid by h_wm in the same way).
// ---------------------------------------------------------------------------
__global__ void k_eqwm_batch(int n, const double *u, const double *h, const double *nu, const double *unit, int ncv,
                             double tau_init, double *tau, int *iters) {
    extern __shared__ double sgu[];
    double *ucv = sgu, *ufa = sgu + ncv + 1;  // ucv[1..ncv], ufa[1..ncv+1]
    for (int q = threadIdx.x; q < 2 * ncv + 3; q += blockDim.x) sgu[q] = unit[q];
    __syncthreads();
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double u_les = u[t], h_wm = h[t], mu_lam = nu[t];
    const double kappa = 0.41, Aplus = 17.0, tol = 0.0000001;
    const int max_iter = 100;
    const double tau_lam = mu_lam * u_les / h_wm;
    const double rw = 1.0 / (ucv[1] * h_wm - ufa[1] * h_wm);
    double tw = tau_init;
    int iter = 0;
    while (true) {
        const double tau_prev = tw;
        const double utau = sqrt(tw);
        const double c1 = kappa * utau;
        const double cd = utau / mu_lam / Aplus;
        double al = u_les, be = 0.0;
        double yf = ufa[ncv] * h_wm;
        double D = 1.0 - exp(-(yf * cd));
        double mu_up = mu_lam + c1 * yf * (D * D);
        for (int q = ncv - 1; q >= 2; q--) {
            yf = ufa[q] * h_wm;
            D = 1.0 - exp(-(yf * cd));
            const double mu_q = mu_lam + c1 * yf * (D * D);
            const double sup = mu_up / (ucv[q + 1] * h_wm - ucv[q] * h_wm);
            const double sub = mu_q / (ucv[q] * h_wm - ucv[q - 1] * h_wm);
            const double m = -1.0 * (sup + sub) + sup * be;
            const double rm = 1.0 / m;
            al = -sup * al * rm;
            be = -sub * rm;
            mu_up = mu_q;
        }
        const double sup = mu_up / (ucv[2] * h_wm - ucv[1] * h_wm);
        const double diag = -1.0 * (sup + mu_lam * rw);
        const double x1 = -sup * al / (diag + sup * be);
        tw = mu_lam * (x1 - 0.0) * rw;
        int done = fabs((tw - tau_prev) / tau_lam) < tol;
        if (!done) iter = iter + 1;
        if (iter > max_iter) done = 1;
        if (done) break;
    }
    tau[t] = tw;
    if (iters) iters[t] = iter;
}

// ---------------------------------------------------------------------------
// Training-set statistics: per block the sums, sums of squares, minima and
// maxima of log u, log h, log nu, log tau (FP64), reduced on the host.
// ---------------------------------------------------------------------------
__global__ void k_mlp_stats(int n, const double *u, const double *h, const double *nu, const double *tau, double *part) {
    __shared__ double sh[16][8];
    double s[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0}, lo[4], hi[4];
    for (int c = 0; c < 4; c++) { lo[c] = INFINITY; hi[c] = -INFINITY; }
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        // the logs of the FP32 inputs, as the network sees them
        const float lu = logf((float)u[t]), lh = logf((float)h[t]), ln = logf((float)nu[t]);
        const double v[4] = {(double)lu, (double)lh, (double)ln, (double)(logf((float)tau[t]) - (ln + lu - lh))};
        for (int c = 0; c < 4; c++) {
            s[c] += v[c];
            q[c] += v[c] * v[c];
            lo[c] = fmin(lo[c], v[c]);
            hi[c] = fmax(hi[c], v[c]);
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = 0; c < 4; c++) {
        for (int o = 16; o > 0; o >>= 1) {
            s[c] += __shfl_down_sync(0xffffffffu, s[c], o);
            q[c] += __shfl_down_sync(0xffffffffu, q[c], o);
            lo[c] = fmin(lo[c], __shfl_down_sync(0xffffffffu, lo[c], o));
            hi[c] = fmax(hi[c], __shfl_down_sync(0xffffffffu, hi[c], o));
        }
    }
    if (lane == 0)
        for (int c = 0; c < 4; c++) {
            sh[4 * c + 0][w] = s[c];
            sh[4 * c + 1][w] = q[c];
            sh[4 * c + 2][w] = lo[c];
            sh[4 * c + 3][w] = hi[c];
        }
    __syncthreads();
    if (threadIdx.x < 16) {
        const int r = threadIdx.x, kind = r & 3;
        double a = sh[r][0];
        for (int q2 = 1; q2 < (int)(blockDim.x >> 5); q2++)
            a = kind == 2 ? fmin(a, sh[r][q2]) : (kind == 3 ? fmax(a, sh[r][q2]) : a + sh[r][q2]);
        part[blockIdx.x * 16 + r] = a;
    }
}

// ---------------------------------------------------------------------------
// Forward + backward of 128 samples per block on the FP32 pipes; per-block
// partial gradients (and loss) for a deterministic reduction.
// Sample of thread s: idx = (pa * (base + s) + pb) mod n (a permutation of
// 0..n-1 for gcd(pa, n) = 1).
// ---------------------------------------------------------------------------
constexpr int GT = 128, GP = MH + 1;  // threads per block, padded row

struct GradSmem {
    float w[NP];           // parameters, W2 rounded to BF16
    float h1b[GT][GP];     // BF16-rounded layer-1 outputs
    float h2[GT][GP];
    float d2[GT][GP];      // dL/dz2
    float d1[GT][GP];      // dL/dz1
    float x[GT][3];
    float dy[GT];
};

__global__ void __launch_bounds__(GT) k_mlp_grad(const float *__restrict__ wm, MlpNorm nm, int n, long base, long pa,
                                                 long pb, const double *u, const double *h, const double *nu,
                                                 const double *tau, float inv_batch, float *part, double *lpart) {
    extern __shared__ __align__(16) unsigned char smraw[];
    GradSmem &S = *reinterpret_cast<GradSmem *>(smraw);
    for (int p = threadIdx.x; p < NP; p += GT) S.w[p] = (p >= O_W2 && p < O_B2) ? bf16r(wm[p]) : wm[p];
    __syncthreads();
    const int s = threadIdx.x;
    const long i = (long)blockIdx.x * GT + s + base;
    const long idx = (long)((unsigned long long)(pa * i + pb) % (unsigned long long)n);
    float x[3];
    const float llam = mlp_features(nm, u[idx], h[idx], nu[idx], x, nullptr);
    const float tgt = (logf((float)tau[idx]) - llam - nm.m[3]) * nm.r[3];
    float a[MH];  // h1 (BF16-rounded), later dL/dz2
#pragma unroll
    for (int k = 0; k < MH; k++) {
        const float z = S.w[O_B1 + k] + S.w[O_W1 + 3 * k] * x[0] + S.w[O_W1 + 3 * k + 1] * x[1] + S.w[O_W1 + 3 * k + 2] * x[2];
        a[k] = bf16r(tanhf(z));
        S.h1b[s][k] = a[k];
    }
    float z2[MH];
#pragma unroll 4
    for (int nn = 0; nn < MH; nn++) {
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < MH; k++) acc = fmaf(S.w[O_W2 + MH * nn + k], a[k], acc);
        z2[nn] = tanhf(acc + S.w[O_B2 + nn]);
    }
    float y = 0.f;
#pragma unroll
    for (int nn = 0; nn < MH; nn++) y = fmaf(S.w[O_W3 + nn], z2[nn], y);
    y += S.w[O_B3];
    const float e = y - tgt;
    const float dy = 2.f * e * inv_batch;
    S.dy[s] = dy;
    S.x[s][0] = x[0];
    S.x[s][1] = x[1];
    S.x[s][2] = x[2];
#pragma unroll
    for (int nn = 0; nn < MH; nn++) {
        S.h2[s][nn] = z2[nn];
        a[nn] = dy * S.w[O_W3 + nn] * (1.f - z2[nn] * z2[nn]);  // dL/dz2
        S.d2[s][nn] = a[nn];
    }
    // dL/dz1 = (W2^T dL/dz2) (1 - h1^2), h1 recomputed in FP32
#pragma unroll 4
    for (int k = 0; k < MH; k++) {
        float acc = 0.f;
#pragma unroll
        for (int nn = 0; nn < MH; nn++) acc = fmaf(S.w[O_W2 + MH * nn + k], a[nn], acc);
        const float z = S.w[O_B1 + k] + S.w[O_W1 + 3 * k] * x[0] + S.w[O_W1 + 3 * k + 1] * x[1] + S.w[O_W1 + 3 * k + 2] * x[2];
        const float t1 = tanhf(z);
        S.d1[s][k] = acc * (1.f - t1 * t1);
    }
    // loss partial
    __shared__ double lw[GT / 32];
    double l = (double)e * (double)e;
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
    if ((s & 31) == 0) lw[s >> 5] = l;
    __syncthreads();
    // per-block sums over the 128 samples
    float *out = part + (long)blockIdx.x * NP;
    for (int p = s; p < MH * MH; p += GT) {  // dW2[nn][k] = sum dz2[nn] h1b[k]
        const int nn = p / MH, k = p % MH;
        float acc = 0.f;
        for (int r = 0; r < GT; r++) acc = fmaf(S.d2[r][nn], S.h1b[r][k], acc);
        out[O_W2 + p] = acc;
    }
    if (s < MH) {
        float b2 = 0.f, w3 = 0.f, b1 = 0.f, w10 = 0.f, w11 = 0.f, w12 = 0.f;
        for (int r = 0; r < GT; r++) {
            b2 += S.d2[r][s];
            w3 = fmaf(S.dy[r], S.h2[r][s], w3);
            const float d = S.d1[r][s];
            b1 += d;
            w10 = fmaf(d, S.x[r][0], w10);
            w11 = fmaf(d, S.x[r][1], w11);
            w12 = fmaf(d, S.x[r][2], w12);
        }
        out[O_B2 + s] = b2;
        out[O_W3 + s] = w3;
        out[O_B1 + s] = b1;
        out[O_W1 + 3 * s] = w10;
        out[O_W1 + 3 * s + 1] = w11;
        out[O_W1 + 3 * s + 2] = w12;
    } else if (s == MH) {
        float b3 = 0.f;
        for (int r = 0; r < GT; r++) b3 += S.dy[r];
        out[O_B3] = b3;
        lpart[blockIdx.x] = lw[0] + lw[1] + lw[2] + lw[3];
    }
}

// sum of the block partials (fixed order) and, if lr > 0, the Adam update;
// thread 0 adds the batch's loss partials to *lacc
__global__ void k_mlp_adam(float *w, float *m1, float *m2, const float *part, int nblk, double *grad_out, float lr,
                           float b1, float b2, float eps, float bc1, float bc2, const double *lpart, double *lacc) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0 && lacc) {
        double l = 0.0;
        for (int b = 0; b < nblk; b++) l += lpart[b];
        *lacc += l;
    }
    if (p >= NP) return;
    double g = 0.0;
    for (int b = 0; b < nblk; b++) g += (double)part[(long)b * NP + p];
    if (grad_out) grad_out[p] = g;
    if (lr <= 0.f) return;
    const float gf = (float)g;
    const float a = b1 * m1[p] + (1.f - b1) * gf, v = b2 * m2[p] + (1.f - b2) * gf * gf;
    m1[p] = a;
    m2[p] = v;
    w[p] -= lr * (a / bc1) / (sqrtf(v / bc2) + eps);
}

// ---------------------------------------------------------------------------
// Inference on the FP32 pipes (the cross-check of the tensor-core kernel).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float mlp_out_to_tau_log(const MlpNorm &nm, float y, float llam) { return y * nm.s3 + nm.m[3] + llam; }

// h and nu are read at t * hs and t * ns (stride 0: one value for all)
__global__ void __launch_bounds__(128) k_mlp_infer_cc(const float *__restrict__ wm, MlpNorm nm, int n, const double *u,
                                                      const double *h, int hs, const double *nu, int ns, double *tau,
                                                      int *inside) {
    __shared__ float w[NP];
    for (int p = threadIdx.x; p < NP; p += blockDim.x) w[p] = (p >= O_W2 && p < O_B2) ? bf16r(wm[p]) : wm[p];
    __syncthreads();
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float x[3];
    bool in;
    const float llam = mlp_features(nm, u[t], h[t * hs], nu[t * ns], x, &in);
    float a[MH];
#pragma unroll
    for (int k = 0; k < MH; k++)
        a[k] = bf16r(tanhf(w[O_B1 + k] + w[O_W1 + 3 * k] * x[0] + w[O_W1 + 3 * k + 1] * x[1] + w[O_W1 + 3 * k + 2] * x[2]));
    float y = 0.f;
#pragma unroll 4
    for (int nn = 0; nn < MH; nn++) {
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < MH; k++) acc = fmaf(w[O_W2 + MH * nn + k], a[k], acc);
        y = fmaf(w[O_W3 + nn], tanhf(acc + w[O_B2 + nn]), y);
    }
    y += w[O_B3];
    tau[t] = exp((double)mlp_out_to_tau_log(nm, y, llam));
    if (inside) inside[t] = in ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Tensor-core inference.  A CTA of 128 threads takes tiles of 128 samples:
// each thread forms its sample's layer-1 activations on the FP32 pipes and
// writes them as one BF16 row of the A tile; one elected thread issues layer
// 2 as four tcgen05.mma (M = 128, N = 64, K = 16 each; A and B BF16, both
// K-major with the 128-byte swizzle; FP32 accumulator in 64 columns of
// tensor memory) and commits them to an mbarrier; every warp then reads its
// 32 accumulator rows (tcgen05.ld 32x32b) and finishes layer 3 in FP32.
// Waits are bounded: on expiry the CTA records an error and stops.
// ---------------------------------------------------------------------------
constexpr int TC_M = 128, TC_N = 64, TC_K = 64;
constexpr uint32_t TC_IDESC = (1u << 4)                  // D: FP32
                              | (1u << 7) | (1u << 10)    // A, B: BF16
                              | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
constexpr long TC_WAIT_LIMIT = 1L << 22;

struct TcSmem {
    unsigned char a[TC_M * TC_K * 2];  // 16 KB, 1024-aligned
    unsigned char b[TC_N * TC_K * 2];  // 8 KB
    float w1[MH * 3], b1[MH], b2[MH], w3[MH], b3;
    unsigned long long mbar;
    unsigned int tmem;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (the leading offset is unused in this mode)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// byte offset of 16-byte chunk c of row r in a K-major tile of 64 BF16 per
// row with the 128-byte swizzle
__device__ __forceinline__ uint32_t sw128_off(int r, int c) { return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4)); }

__device__ __forceinline__ uint4 pack8_bf16(const float *v) {
    uint4 q;
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]), p1 = __floats2bfloat162_rn(v[2], v[3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(v[4], v[5]), p3 = __floats2bfloat162_rn(v[6], v[7]);
    q.x = *reinterpret_cast<uint32_t *>(&p0);
    q.y = *reinterpret_cast<uint32_t *>(&p1);
    q.z = *reinterpret_cast<uint32_t *>(&p2);
    q.w = *reinterpret_cast<uint32_t *>(&p3);
    return q;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

// a wait gives up after TC_WAIT_NS nanoseconds or TC_WAIT_LIMIT polls,
// whichever comes first (a completed MMA arrives within microseconds)
constexpr uint64_t TC_WAIT_NS = 1000000000ull;

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t phase) {
    const uint64_t t0 = global_ns();
    for (long it = 0; it < TC_WAIT_LIMIT; it++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(addr), "r"(phase)
            : "memory");
        if (ok) return true;
        if ((it & 63) == 63 && global_ns() - t0 > TC_WAIT_NS) return false;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

__global__ void __launch_bounds__(TC_M) k_mlp_infer_tc(const float *__restrict__ wm, MlpNorm nm, int n, const double *u,
                                                       const double *h, int hs, const double *nu, int ns, double *tau,
                                                       int *inside, int *err, int skip_mma) {
    extern __shared__ unsigned char tc_raw[];
    // 1024-byte alignment of the tiles (the swizzle pattern is anchored to it)
    const uint32_t raw = smem_u32(tc_raw);
    TcSmem &S = *reinterpret_cast<TcSmem *>(tc_raw + (((raw + 1023u) & ~1023u) - raw));
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t a_addr = smem_u32(S.a), b_addr = smem_u32(S.b), mbar = smem_u32(&S.mbar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&S.tmem)),
                     "r"(TC_N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // W2 as the B tile (row n = output unit, K-major), BF16
    for (int q = tid; q < TC_N * 8; q += TC_M) {
        const int r = q >> 3, c = q & 7;
        *reinterpret_cast<uint4 *>(S.b + sw128_off(r, c)) = pack8_bf16(wm + O_W2 + MH * r + 8 * c);
    }
    for (int q = tid; q < MH * 3; q += TC_M) S.w1[q] = wm[O_W1 + q];
    for (int q = tid; q < MH; q += TC_M) {
        S.b1[q] = wm[O_B1 + q];
        S.b2[q] = wm[O_B2 + q];
        S.w3[q] = wm[O_W3 + q];
    }
    if (tid == 0) S.b3 = wm[O_B3];
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = S.tmem;
    uint32_t phase = 0;
    const int ntiles = (n + TC_M - 1) / TC_M;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long s = (long)tile * TC_M + tid;
        const bool valid = s < n;
        float x[3] = {0.f, 0.f, 0.f}, llam = 0.f;
        bool in = false;
        if (valid) llam = mlp_features(nm, u[s], h[s * hs], nu[s * ns], x, &in);
        // layer 1 -> BF16 row tid of the A tile
#pragma unroll
        for (int c = 0; c < 8; c++) {
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int k = 8 * c + e;
                v[e] = tanhf(S.b1[k] + S.w1[3 * k] * x[0] + S.w1[3 * k + 1] * x[1] + S.w1[3 * k + 2] * x[2]);
            }
            *reinterpret_cast<uint4 *>(S.a + sw128_off(tid, c)) = pack8_bf16(v);
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0 && !skip_mma) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int kk = 0; kk < TC_K / 16; kk++) {
                const uint64_t ad = sw128_desc(a_addr + 32u * kk), bd = sw128_desc(b_addr + 32u * kk);
                const uint32_t acc = kk > 0 ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(TC_IDESC), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                         : "memory");
        }
        const bool ok = mbar_wait(mbar, phase);
        if (__syncthreads_or(!ok)) {
            // The commit did not arrive in time.  Record it, give the MMA of
            // this tile (if one was issued) a second bounded wait before its
            // tensor memory is freed below, and mark every sample of this
            // block's remaining tiles as not served, so that a caller that
            // falls back outside the envelope (the wall model) solves eqwm
            // there.
            if (tid == 0) atomicExch(err, 1);
            if (!ok) mbar_wait(mbar, phase);
            if (inside)
                for (int t2 = tile; t2 < ntiles; t2 += gridDim.x) {
                    const long s2 = (long)t2 * TC_M + tid;
                    if (s2 < n) inside[s2] = 0;
                }
            break;
        }
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        float acc[TC_N];
        const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll
        for (int q = 0; q < TC_N / 16; q++) tmem_ld16(trow + 16u * q, acc + 16 * q);
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        float y = 0.f;
#pragma unroll
        for (int nn = 0; nn < TC_N; nn++) y = fmaf(S.w3[nn], tanhf(acc[nn] + S.b2[nn]), y);
        y += S.b3;
        if (valid) {
            tau[s] = exp((double)mlp_out_to_tau_log(nm, y, llam));
            if (inside) inside[s] = in ? 1 : 0;
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();  // accumulator read and A tile free for the next tile
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC_N));
}

// ---------------------------------------------------------------------------
// Forward + backward of 128 samples per CTA with the three 64-wide products
// of layer 2 on the tensor cores (tcgen05.mma kind::f16, BF16 operands, FP32
// accumulators in tensor memory), the rest on the FP32 pipes:
//   MMA1  z2  = H1b W2^T        A = H1b [s][k],    B = W2 [nn][k]      -> cols   0..63
//   MMA2  dh1 = D2b W2          A = D2b [s][nn],   B = W2^T [k][nn]    -> cols  64..127
//   MMA3  dW2 = D2b^T H1b       A = D2b^T [nn][s] (rows 64..127 zero),
//                               B = H1b^T [k][s]   (K = 128 samples)   -> cols 128..191
// H1b = the BF16 layer-1 outputs, D2b = dL/dz2 rounded to BF16 (the products
// that feed a tensor-core MMA take BF16 operands; the bias and layer-1/3
// gradients use the FP32 dL/dz2).  Every operand tile is K-major with the
// 128-byte swizzle: rows of 64 BF16 (128 B), 8-row groups 1024 B apart, a
// K of 128 as two such tiles.  Thread s owns sample s = tensor-memory lane s.
// Waits are bounded as in the inference; on expiry the CTA records it and
// writes no gradient.
// ---------------------------------------------------------------------------
struct GradTcSmem {
    unsigned char a1[128 * 128];      // H1b [s][k]
    unsigned char a2[128 * 128];      // D2b [s][nn]
    unsigned char a3[2][128 * 128];   // D2b^T [nn][s], K halves s < 64, s >= 64
    unsigned char tb3[2][64 * 128];   // H1b^T [k][s], K halves
    unsigned char b2f[64 * 128];      // W2 [nn][k]
    unsigned char b2b[64 * 128];      // W2^T [k][nn]
    float h2[GT][GP];                 // h2 (for the W3 gradient)
    float d2[GT][GP];                 // FP32 dL/dz2 (b2 gradient)
    float d1[GT][GP];                 // dL/dz1
    float x[GT][3];
    float dy[GT];
    float w1[MH * 3], b1[MH], b2[MH], w3[MH], b3;
    double lw[GT / 32];
    unsigned long long mbar;
    unsigned int tmem;
};

// byte offset of element (row r, K index c) in a K-major 128B-swizzled tile
// of 64-element rows
__device__ __forceinline__ uint32_t sw128_elem(int r, int c) { return sw128_off(r, c >> 3) + 2u * (uint32_t)(c & 7); }

__device__ __forceinline__ void put_bf16(unsigned char *tile, int r, int c, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(tile + sw128_elem(r, c)) = __float2bfloat16_rn(v);
}

// one K-major MMA group: nk slices of K = 16 from A (tiles of 128 rows,
// 16 KB apart per 64 K) and B (tiles of 64 rows, 8 KB apart per 64 K)
__device__ __forceinline__ void mma_k(uint32_t tmem_d, uint32_t a0, uint32_t b0, int nk) {
    for (int kk = 0; kk < nk; kk++) {
        const uint32_t ah = a0 + (uint32_t)(kk >> 2) * (128u * 128u) + 32u * (kk & 3);
        const uint32_t bh = b0 + (uint32_t)(kk >> 2) * (64u * 128u) + 32u * (kk & 3);
        const uint64_t ad = sw128_desc(ah), bd = sw128_desc(bh);
        const uint32_t acc = kk > 0 ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
            "l"(ad), "l"(bd), "r"(TC_IDESC), "r"(acc));
    }
}

__global__ void __launch_bounds__(GT) k_mlp_grad_tc(const float *__restrict__ wm, MlpNorm nm, int n, long base, long pa,
                                                    long pb, const double *u, const double *h, const double *nu,
                                                    const double *tau, float inv_batch, float *part, double *lpart,
                                                    int *err) {
    extern __shared__ unsigned char tc_raw[];
    const uint32_t raw = smem_u32(tc_raw);
    GradTcSmem &S = *reinterpret_cast<GradTcSmem *>(tc_raw + (((raw + 1023u) & ~1023u) - raw));
    const int s = threadIdx.x, warp = s >> 5;
    const uint32_t mbar = smem_u32(&S.mbar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&S.tmem)),
                     "r"(256));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (s == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // W2 as B of MMA1 (K-major rows nn) and, transposed, of MMA2 (rows k)
    for (int q = s; q < MH * 8; q += GT) {
        const int r = q >> 3, c = q & 7;
        *reinterpret_cast<uint4 *>(S.b2f + sw128_off(r, c)) = pack8_bf16(wm + O_W2 + MH * r + 8 * c);
    }
    for (int q = s; q < MH * MH; q += GT) {
        const int nn = q / MH, k = q % MH;
        put_bf16(S.b2b, k, nn, wm[O_W2 + q]);
    }
    // rows 64..127 of D2b^T stay zero
    for (int q = s; q < 2 * 64 * 8; q += GT) {
        const int hf = q / (64 * 8), r = 64 + (q / 8) % 64, c = q & 7;
        *reinterpret_cast<uint4 *>(S.a3[hf] + sw128_off(r, c)) = make_uint4(0u, 0u, 0u, 0u);
    }
    for (int q = s; q < MH * 3; q += GT) S.w1[q] = wm[O_W1 + q];
    for (int q = s; q < MH; q += GT) {
        S.b1[q] = wm[O_B1 + q];
        S.b2[q] = wm[O_B2 + q];
        S.w3[q] = wm[O_W3 + q];
    }
    if (s == 0) S.b3 = wm[O_B3];
    // layer 1 of sample s
    const long i = (long)blockIdx.x * GT + s + base;
    const long idx = (long)((unsigned long long)(pa * i + pb) % (unsigned long long)n);
    float x[3];
    const float llam = mlp_features(nm, u[idx], h[idx], nu[idx], x, nullptr);
    const float tgt = (logf((float)tau[idx]) - llam - nm.m[3]) * nm.r[3];
    __syncthreads();  // parameters staged
#pragma unroll
    for (int c = 0; c < 8; c++) {
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; e++) {
            const int k = 8 * c + e;
            v[e] = tanhf(S.b1[k] + S.w1[3 * k] * x[0] + S.w1[3 * k + 1] * x[1] + S.w1[3 * k + 2] * x[2]);
        }
        *reinterpret_cast<uint4 *>(S.a1 + sw128_off(s, c)) = pack8_bf16(v);
#pragma unroll
        for (int e = 0; e < 8; e++) put_bf16(S.tb3[s >> 6], 8 * c + e, s & 63, v[e]);
    }
    S.x[s][0] = x[0];
    S.x[s][1] = x[1];
    S.x[s][2] = x[2];
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = S.tmem;
    if (s == 0) {
        mma_k(tmem, smem_u32(S.a1), smem_u32(S.b2f), 4);
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                     : "memory");
    }
    bool ok = mbar_wait(mbar, 0u);
    if (__syncthreads_or(!ok)) {
        if (s == 0) atomicExch(err, 1);
        if (!ok) mbar_wait(mbar, 0u);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);
        float z[MH];
#pragma unroll
        for (int q = 0; q < MH / 16; q++) tmem_ld16(trow + 16u * q, z + 16 * q);
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        float y = 0.f;
#pragma unroll
        for (int nn = 0; nn < MH; nn++) {
            z[nn] = tanhf(z[nn] + S.b2[nn]);  // h2
            y = fmaf(S.w3[nn], z[nn], y);
        }
        y += S.b3;
        const float e = y - tgt;
        const float dy = 2.f * e * inv_batch;
        S.dy[s] = dy;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            float v[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int nn = 8 * c + q;
                S.h2[s][nn] = z[nn];
                v[q] = dy * S.w3[nn] * (1.f - z[nn] * z[nn]);  // dL/dz2
                S.d2[s][nn] = v[q];
                put_bf16(S.a3[s >> 6], nn, s & 63, v[q]);
            }
            *reinterpret_cast<uint4 *>(S.a2 + sw128_off(s, c)) = pack8_bf16(v);
        }
        double l = (double)e * (double)e;
        for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
        if ((s & 31) == 0) S.lw[warp] = l;
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (s == 0) {
            mma_k(tmem + 64u, smem_u32(S.a2), smem_u32(S.b2b), 4);
            mma_k(tmem + 128u, smem_u32(S.a3[0]), smem_u32(S.tb3[0]), 8);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                         : "memory");
        }
        ok = mbar_wait(mbar, 1u);
        if (__syncthreads_or(!ok)) {
            if (s == 0) atomicExch(err, 1);
            if (!ok) mbar_wait(mbar, 1u);
        } else {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            float g[MH];
#pragma unroll
            for (int q = 0; q < MH / 16; q++) tmem_ld16(trow + 64u + 16u * q, g + 16 * q);
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            // dL/dz1 = (dL/dz2 W2) (1 - h1^2), h1 recomputed in FP32
#pragma unroll
            for (int k = 0; k < MH; k++) {
                const float t1 = tanhf(S.b1[k] + S.w1[3 * k] * x[0] + S.w1[3 * k + 1] * x[1] + S.w1[3 * k + 2] * x[2]);
                S.d1[s][k] = g[k] * (1.f - t1 * t1);
            }
            float *out = part + (long)blockIdx.x * NP;
            if (warp < 2) {  // lanes 0..63 hold dW2[nn][k], nn = lane
#pragma unroll
                for (int q = 0; q < MH / 16; q++) tmem_ld16(trow + 128u + 16u * q, g + 16 * q);
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                for (int k = 0; k < MH; k++) out[O_W2 + MH * s + k] = g[k];
            }
            __syncthreads();
            if (s < MH) {
                float b2 = 0.f, w3 = 0.f, b1 = 0.f, w10 = 0.f, w11 = 0.f, w12 = 0.f;
                for (int r = 0; r < GT; r++) {
                    b2 += S.d2[r][s];
                    w3 = fmaf(S.dy[r], S.h2[r][s], w3);
                    const float d = S.d1[r][s];
                    b1 += d;
                    w10 = fmaf(d, S.x[r][0], w10);
                    w11 = fmaf(d, S.x[r][1], w11);
                    w12 = fmaf(d, S.x[r][2], w12);
                }
                out[O_B2 + s] = b2;
                out[O_W3 + s] = w3;
                out[O_B1 + s] = b1;
                out[O_W1 + 3 * s] = w10;
                out[O_W1 + 3 * s + 1] = w11;
                out[O_W1 + 3 * s + 2] = w12;
            } else if (s == MH) {
                float b3 = 0.f;
                for (int r = 0; r < GT; r++) b3 += S.dy[r];
                out[O_B3] = b3;
                lpart[blockIdx.x] = S.lw[0] + S.lw[1] + S.lw[2] + S.lw[3];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(256));
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct cf_mlp {
    int dev = 0, ncv = 0, sms = 152;
    int *derr = nullptr;  // set by a tensor-core wait that expired
    int test_skip_mma = 0;  // test hook: the inference issues no MMA, so its waits expire
    int train_tc = 1;       // gradients with layer 2 on the tensor cores (0: FP32 pipes)
    double stretch = 0.0;
    float *w = nullptr, *m1 = nullptr, *m2 = nullptr, *part = nullptr;
    double *lpart = nullptr, *unit = nullptr;
    int part_blocks = 0;
    long step = 0;
    double norm[8] = {0, 0, 0, 0, 1, 1, 1, 1}, env[6] = {-1e30, -1e30, -1e30, 1e30, 1e30, 1e30};
    std::string err;
};

static thread_local std::string g_mlp_err;
static int mlp_fail(cf_mlp *m, int code, const std::string &msg) {
    if (m) m->err = msg;
    g_mlp_err = msg;
    return code;
}
#define MLP_CUDA(call)                                                                             \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return mlp_fail(m, CF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static MlpNorm norm_of(const cf_mlp *m) {
    MlpNorm nm;
    for (int c = 0; c < 4; c++) {
        nm.m[c] = (float)m->norm[c];
        nm.r[c] = (float)(1.0 / m->norm[4 + c]);
    }
    nm.s3 = (float)m->norm[7];
    for (int c = 0; c < 3; c++) {
        nm.lo[c] = (float)m->env[c];
        nm.hi[c] = (float)m->env[3 + c];
    }
    return nm;
}

// the ODE grid of eqwm.f90:20-50 for h_wm = 1: ucv[1..ncv], ufa[1..ncv+1]
static std::vector<double> unit_grid(int ncv, double stretch) {
    std::vector<double> cv(ncv + 2, 0.0), fa(ncv + 2, 0.0);
    fa[1] = 0.0;
    double inc = 1.0;
    for (int i = 2; i <= ncv + 1; i++) {
        fa[i] = fa[i - 1] + inc;
        cv[i - 1] = 0.5 * (fa[i] + fa[i - 1]);
        inc = inc * stretch;
    }
    double ymax = cv[1];
    for (int i = 1; i <= ncv; i++) ymax = std::max(ymax, cv[i]);
    std::vector<double> out(2 * ncv + 3, 0.0);
    for (int i = 1; i <= ncv; i++) out[i] = cv[i] / ymax * 1.0;
    for (int i = 1; i <= ncv + 1; i++) out[ncv + 1 + i] = fa[i] / ymax * 1.0;  // ufa[i] at sgu[ncv+1+i]
    return out;
}

extern "C" int cf_eqwm_solve_batch(int n, const double *u, const double *h, const double *nu, int ncv, double stretch,
                                   double tau_init, double *tau, int *iters, void *stream) {
    cf_mlp *m = nullptr;
    if (n < 0 || !u || !h || !nu || !tau || ncv < 3 || ncv > 2048 || !(stretch > 0))
        return mlp_fail(m, CF_ERR_INVALID, "cf_eqwm_solve_batch: bad argument");
    if (n == 0) return CF_OK;
    std::vector<double> g = unit_grid(ncv, stretch);
    double *dg;
    MLP_CUDA(cudaMalloc(&dg, g.size() * sizeof(double)));
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(dg, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_eqwm_batch<<<cdiv(n, 128), 128, g.size() * sizeof(double), st>>>(n, u, h, nu, dg, ncv, tau_init, tau, iters);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dg);
    if (e != cudaSuccess) return mlp_fail(m, CF_ERR_CUDA, std::string("cf_eqwm_solve_batch: ") + cudaGetErrorString(e));
    return CF_OK;
}

extern "C" int cf_mlp_create(int seed, int ncv, double stretch, cf_mlp **out) {
    cf_mlp *m = nullptr;
    if (!out || ncv < 3 || !(stretch > 0)) return mlp_fail(m, CF_ERR_INVALID, "cf_mlp_create: bad argument");
    *out = nullptr;
    m = new cf_mlp();
    m->ncv = ncv;
    m->stretch = stretch;
    cudaGetDevice(&m->dev);
    // Xavier-uniform weights, zero biases (seeded LCG; the host draws them)
    std::vector<float> w(NP, 0.f);
    unsigned long long st = 0x9E3779B97F4A7C15ull * (unsigned long long)(seed + 1);
    auto uni = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return (double)(st >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int cnt, int fan_in, int fan_out) {
        const double a = std::sqrt(6.0 / (fan_in + fan_out));
        for (int q = 0; q < cnt; q++) w[off + q] = (float)((2.0 * uni() - 1.0) * a);
    };
    fill(O_W1, 3 * MH, 3, MH);
    fill(O_W2, MH * MH, MH, MH);
    fill(O_W3, MH, MH, 1);
    cudaError_t e = cudaMalloc(&m->w, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->m1, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->m2, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(m->w, w.data(), NP * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->m1, 0, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->m2, 0, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GradSmem));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_grad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GradTcSmem) + 1024);
    if (e == cudaSuccess) e = cudaMalloc(&m->derr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(m->derr, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, m->dev);
    if (e != cudaSuccess) {
        int rc = mlp_fail(m, CF_ERR_CUDA, std::string("cf_mlp_create: ") + cudaGetErrorString(e));
        cf_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return CF_OK;
}

extern "C" int cf_mlp_destroy(cf_mlp *m) {
    if (!m) return CF_OK;
    void *p[] = {m->w, m->m1, m->m2, m->part, m->lpart, m->unit, m->derr};
    for (void *q : p)
        if (q) cudaFree(q);
    delete m;
    return CF_OK;
}

extern "C" int cf_mlp_fit_normalisation(cf_mlp *m, int n, const double *u, const double *h, const double *nu,
                                        const double *tau, void *stream) {
    if (!m || n < 2 || !u || !h || !nu || !tau) return mlp_fail(m, CF_ERR_INVALID, "cf_mlp_fit_normalisation: bad argument");
    const int nb = 256;
    double *d;
    MLP_CUDA(cudaMalloc(&d, nb * 16 * sizeof(double)));
    cudaStream_t st = (cudaStream_t)stream;
    k_mlp_stats<<<nb, 256, 0, st>>>(n, u, h, nu, tau, d);
    std::vector<double> r(nb * 16);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.data(), d, r.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) return mlp_fail(m, CF_ERR_CUDA, std::string("cf_mlp_fit_normalisation: ") + cudaGetErrorString(e));
    for (int c = 0; c < 4; c++) {
        double s = 0, q = 0, lo = INFINITY, hi = -INFINITY;
        for (int b = 0; b < nb; b++) {
            s += r[b * 16 + 4 * c];
            q += r[b * 16 + 4 * c + 1];
            lo = std::min(lo, r[b * 16 + 4 * c + 2]);
            hi = std::max(hi, r[b * 16 + 4 * c + 3]);
        }
        const double mean = s / n, var = std::max(q / n - mean * mean, 1e-30);
        m->norm[c] = mean;
        m->norm[4 + c] = std::sqrt(var);
        if (c < 3) {
            m->env[c] = lo;
            m->env[3 + c] = hi;
        }
    }
    return CF_OK;
}

static int ensure_part(cf_mlp *m, int nblk) {
    if (m->part_blocks >= nblk) return 0;
    if (m->part) cudaFree(m->part);
    if (m->lpart) cudaFree(m->lpart);
    m->part = nullptr;
    m->lpart = nullptr;
    MLP_CUDA(cudaMalloc(&m->part, (size_t)nblk * NP * sizeof(float)));
    MLP_CUDA(cudaMalloc(&m->lpart, (size_t)(nblk + 1) * sizeof(double)));
    m->part_blocks = nblk;
    return 0;
}

static long gcdl(long a, long b) { return b == 0 ? a : gcdl(b, a % b); }

// per-block partial gradients of nblk tiles of 128 samples
static void launch_grad(cf_mlp *m, int nblk, const MlpNorm &nm, int n, long base, long pa, long pb, const double *u,
                        const double *h, const double *nu, const double *tau, float inv_batch, cudaStream_t st) {
    if (m->train_tc)
        k_mlp_grad_tc<<<nblk, GT, sizeof(GradTcSmem) + 1024, st>>>(m->w, nm, n, base, pa, pb, u, h, nu, tau, inv_batch,
                                                                    m->part, m->lpart, m->derr);
    else
        k_mlp_grad<<<nblk, GT, sizeof(GradSmem), st>>>(m->w, nm, n, base, pa, pb, u, h, nu, tau, inv_batch, m->part,
                                                         m->lpart);
}

extern "C" int cf_mlp_set_train_tensor_cores(cf_mlp *m, int on) {
    if (!m) return mlp_fail(m, CF_ERR_INVALID, "cf_mlp_set_train_tensor_cores: null network");
    m->train_tc = on ? 1 : 0;
    return CF_OK;
}

extern "C" int cf_mlp_gradient(cf_mlp *m, int n, const double *u, const double *h, const double *nu,
                               const double *tau, double *grad, double *loss, void *stream) {
    if (!m || n < GT || n % GT || !u || !h || !nu || !tau || !grad)
        return mlp_fail(m, CF_ERR_INVALID, "cf_mlp_gradient: n must be a positive multiple of 128");
    const int nblk = n / GT;
    if (int rc = ensure_part(m, nblk)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    launch_grad(m, nblk, norm_of(m), n, 0, 1, 0, u, h, nu, tau, 1.f / n, st);
    k_mlp_adam<<<cdiv(NP, 256), 256, 0, st>>>(m->w, m->m1, m->m2, m->part, nblk, grad, 0.f, 0.f, 0.f, 0.f, 1.f, 1.f,
                                               nullptr, nullptr);
    MLP_CUDA(cudaGetLastError());
    if (loss) {
        std::vector<double> l(nblk);
        MLP_CUDA(cudaMemcpyAsync(l.data(), m->lpart, nblk * sizeof(double), cudaMemcpyDeviceToHost, st));
        MLP_CUDA(cudaStreamSynchronize(st));
        double s = 0;
        for (double v : l) s += v;
        *loss = s / n;
    }
    MLP_CUDA(cudaStreamSynchronize(st));
    return CF_OK;
}

extern "C" int cf_mlp_train(cf_mlp *m, int n, const double *u, const double *h, const double *nu, const double *tau,
                            int epochs, int batch, double lr, int seed, double *loss_out, void *stream) {
    if (!m || batch < GT || batch % GT || n < batch || epochs < 1 || !(lr > 0) || !u || !h || !nu || !tau)
        return mlp_fail(m, CF_ERR_INVALID, "cf_mlp_train: bad argument (batch a multiple of 128, n >= batch)");
    const int nblk = batch / GT, nbatch = n / batch;
    if (int rc = ensure_part(m, nblk)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const MlpNorm nm = norm_of(m);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const long total = (long)epochs * nbatch;
    unsigned long long rs = 0xD1B54A32D192ED03ull * (unsigned long long)(seed + 7);
    auto rnd = [&]() {
        rs = rs * 6364136223846793005ull + 1442695040888963407ull;
        return (long)(rs >> 17);
    };
    double *lacc = m->lpart + nblk;  // per-epoch loss sum (ensure_part leaves room)
    for (int ep = 0; ep < epochs; ep++) {
        MLP_CUDA(cudaMemsetAsync(lacc, 0, sizeof(double), st));
        // a seeded affine permutation of the samples per epoch
        long pa;
        do {
            pa = (rnd() % (long)n) | 1;
        } while (gcdl(pa, n) != 1);
        const long pb = rnd() % (long)n;
        for (int bt = 0; bt < nbatch; bt++) {
            const long k = (long)ep * nbatch + bt;
            const double lr_t = lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(3.141592653589793 * (double)k / (double)total)));
            m->step++;
            const float bc1 = 1.f - std::pow(b1, (float)m->step), bc2 = 1.f - std::pow(b2, (float)m->step);
            launch_grad(m, nblk, nm, n, (long)bt * batch, pa, pb, u, h, nu, tau, 1.f / batch, st);
            k_mlp_adam<<<cdiv(NP, 256), 256, 0, st>>>(m->w, m->m1, m->m2, m->part, nblk, nullptr, (float)lr_t, b1,
                                                        b2, eps, bc1, bc2, m->lpart, lacc);
        }
        MLP_CUDA(cudaGetLastError());
        if (loss_out) {
            double lsum = 0.0;
            MLP_CUDA(cudaMemcpyAsync(&lsum, lacc, sizeof(double), cudaMemcpyDeviceToHost, st));
            MLP_CUDA(cudaStreamSynchronize(st));
            loss_out[ep] = lsum / ((double)nbatch * batch);
        }
    }
    MLP_CUDA(cudaStreamSynchronize(st));
    return CF_OK;
}

int mlp_predict_tc(cf_mlp *m, int n, const double *u, const double *h, int hs, const double *nu, int ns, double *tau,
                   int *inside, cudaStream_t st);

extern "C" int cf_mlp_predict(cf_mlp *m, int n, const double *u, const double *h, const double *nu, double *tau,
                              int *inside, int use_tensor_cores, void *stream) {
    if (!m || n < 0 || !u || !h || !nu || !tau) return mlp_fail(m, CF_ERR_INVALID, "cf_mlp_predict: bad argument");
    if (n == 0) return CF_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (use_tensor_cores) {
        if (int rc = mlp_predict_tc(m, n, u, h, 1, nu, 1, tau, inside, st)) return rc;
        int e = 0;
        MLP_CUDA(cudaMemcpyAsync(&e, m->derr, sizeof(int), cudaMemcpyDeviceToHost, st));
        MLP_CUDA(cudaStreamSynchronize(st));
        if (e) {
            MLP_CUDA(cudaMemsetAsync(m->derr, 0, sizeof(int), st));
            return mlp_fail(m, CF_ERR_CUDA, "cf_mlp_predict: a tensor-core wait expired");
        }
    } else {
        k_mlp_infer_cc<<<cdiv(n, 128), 128, 0, st>>>(m->w, norm_of(m), n, u, h, 1, nu, 1, tau, inside);
    }
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaStreamSynchronize(st));
    return CF_OK;
}

extern "C" int cf_mlp_get(cf_mlp *m, float *params, double *norm, double *envelope) {
    if (!m) return mlp_fail(m, CF_ERR_INVALID, "null network");
    if (params) MLP_CUDA(cudaMemcpy(params, m->w, NP * sizeof(float), cudaMemcpyDeviceToHost));
    if (norm) std::copy(m->norm, m->norm + 8, norm);
    if (envelope) std::copy(m->env, m->env + 6, envelope);
    return CF_OK;
}

extern "C" int cf_mlp_set(cf_mlp *m, const float *params, const double *norm, const double *envelope) {
    if (!m) return mlp_fail(m, CF_ERR_INVALID, "null network");
    if (params) MLP_CUDA(cudaMemcpy(m->w, params, NP * sizeof(float), cudaMemcpyHostToDevice));
    if (norm) std::copy(norm, norm + 8, m->norm);
    if (envelope) std::copy(envelope, envelope + 6, m->env);
    return CF_OK;
}

int mlp_predict_tc(cf_mlp *m, int n, const double *u, const double *h, int hs, const double *nu, int ns, double *tau,
                   int *inside, cudaStream_t st) {
    const int ntiles = cdiv(n, TC_M);
    const int grid = std::min(ntiles, m->sms * 4);
    k_mlp_infer_tc<<<grid, TC_M, sizeof(TcSmem) + 1024, st>>>(m->w, norm_of(m), n, u, h, hs, nu, ns, tau, inside,
                                                              m->derr, m->test_skip_mma);
    return 0;
}

extern "C" int cf_mlp_wait_expired(cf_mlp *m, int *expired) {
    if (!m || !expired) return mlp_fail(m, CF_ERR_INVALID, "cf_mlp_wait_expired: null argument");
    MLP_CUDA(cudaSetDevice(m->dev));
    MLP_CUDA(cudaDeviceSynchronize());
    MLP_CUDA(cudaMemcpy(expired, m->derr, sizeof(int), cudaMemcpyDeviceToHost));
    MLP_CUDA(cudaMemset(m->derr, 0, sizeof(int)));
    return CF_OK;
}

extern "C" int cf_mlp_test_skip_mma(cf_mlp *m, int on) {
    if (!m) return mlp_fail(m, CF_ERR_INVALID, "cf_mlp_test_skip_mma: null network");
    m->test_skip_mma = on ? 1 : 0;
    return CF_OK;
}

// ---------------------------------------------------------------------------
// the learned stress in the equilibrium wall model of a context
// ---------------------------------------------------------------------------
int wall_mlp_infer(cf_ctx *ctx, int npts, double h_wm, double nu) {
    (void)h_wm;
    (void)nu;
    // wm_log[6], wm_log[7] hold the matching height and the viscosity
    if (mlp_predict_tc(ctx->wmlp, npts, ctx->wm_u, ctx->wm_log + 6, 0, ctx->wm_log + 7, 0, ctx->wm_tau,
                       ctx->wm_inside, ctx->st))
        return cf_fail(ctx, CF_ERR_CUDA, "learned wall stress: " + ctx->wmlp->err);
    count_launch(ctx, "k_mlp_infer_tc");
    return 0;
}

extern "C" int cf_set_wall_mlp(cf_ctx *ctx, cf_mlp *m, int check_every) {
    if (!ctx) return cf_fail(ctx, CF_ERR_INVALID, "null context");
    if (ctx->prm.iwall_model != 3) return cf_fail(ctx, CF_ERR_INVALID, "the learned wall stress needs iwall_model 3");
    if (check_every < 0) return cf_fail(ctx, CF_ERR_INVALID, "check_every must be >= 0");
    if (m && (m->ncv != ctx->prm.eqwm_ncv || std::fabs(m->stretch - ctx->prm.eqwm_stretch) > 1e-12))
        return cf_fail(ctx, CF_ERR_INVALID, "the network was trained for another eqwm grid (eqwm_ncv, eqwm_stretch)");
    CF_CUDA(cudaSetDevice(ctx->dev));
    CF_CUDA(cudaStreamSynchronize(ctx->st));
    const size_t nwall = (size_t)ctx->nxg * 2 * ctx->nzg;
    if (m && !ctx->wm_u) {
        CF_CUDA(cudaMalloc(&ctx->wm_u, nwall * sizeof(double)));
        CF_CUDA(cudaMalloc(&ctx->wm_tau, nwall * sizeof(double)));
        CF_CUDA(cudaMalloc(&ctx->wm_tau_eq, nwall * sizeof(double)));
        CF_CUDA(cudaMalloc(&ctx->wm_inside, nwall * sizeof(int)));
        CF_CUDA(cudaMalloc(&ctx->wm_calls, sizeof(int)));
        CF_CUDA(cudaMalloc(&ctx->wm_log, 8 * sizeof(double)));
    }
    if (m) {
        double hl[8] = {0, 0, 0, 0, 0, 0, ctx->hyg[ctx->prm.jref_eqwm], ctx->prm.nu};
        CF_CUDA(cudaMemcpy(ctx->wm_log, hl, sizeof(hl), cudaMemcpyHostToDevice));
        CF_CUDA(cudaMemset(ctx->wm_calls, 0, sizeof(int)));
    }
    ctx->wmlp = m;
    ctx->wm_check_every = check_every;
    // the captured steps do not contain the new sequence
    for (auto &g : ctx->graphs)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    return CF_OK;
}

extern "C" int cf_get_wall_mlp_log(cf_ctx *ctx, double *out) {
    if (!ctx || !out) return cf_fail(ctx, CF_ERR_INVALID, "null argument");
    if (!ctx->wm_log) {
        for (int q = 0; q < 5; q++) out[q] = 0.0;
        return CF_OK;
    }
    CF_CUDA(cudaSetDevice(ctx->dev));
    double h[8];
    int calls = 0;
    CF_CUDA(cudaMemcpyAsync(h, ctx->wm_log, sizeof(h), cudaMemcpyDeviceToHost, ctx->st));
    CF_CUDA(cudaMemcpyAsync(&calls, ctx->wm_calls, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CF_CUDA(cudaStreamSynchronize(ctx->st));
    out[0] = calls;
    for (int q = 1; q < 5; q++) out[q] = h[q];
    return CF_OK;
}
