// k_stats.cu -- plane statistics of compute_statistics (statistics.f90:43-159).
// Raw sums go to the host, which applies the reference's normalisations.
// Output layout: 7*ny profile sums (per j: U, V, W, U^2, V^2, W^2, UV), then
// U(1), U(2), U(nyg-1), U(nyg) plane sums, nu_t sums at rows 1:2 and
// nyg-1:nyg, and the U and V trapezoid sums of mass_flow.f90:37-44, 73-80.
#include "cf_internal.cuh"

__device__ __forceinline__ double bsum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffff, v, o);
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) r += sh[q];
    __syncthreads();
    return r;
}

template <typename T>
__global__ void k_stats_prof(Geo g, Fld<T> U, Fld<T> V, Fld<T> W, double *out) {
    __shared__ double sh[32];
    int jj = blockIdx.x + 1;  // 1..ny
    const double w0 = g.w0[jj], w1 = g.w1[jj];
    double su = 0, su2 = 0, sw = 0, sw2 = 0, sv = 0, sv2 = 0, suv = 0;
    // Umean: term_1(1:nx-2, jj, 1:nzg-2)
    long n1 = (long)(g.nx - 2) * (g.nzg - 2);
    for (long t = threadIdx.x; t < n1; t += blockDim.x) {
        int i = (int)(t % (g.nx - 2)) + 1, k = (int)(t / (g.nx - 2)) + 1;
        double t1 = w0 * (double)U(i, jj, k) + w1 * (double)U(i, jj + 1, k);
        su += t1;
        su2 += t1 * t1;
    }
    // Wmean: term_2(1:nxg-2, jj, 1:nz-2)
    long n2 = (long)(g.nxg - 2) * (g.nz - 2);
    for (long t = threadIdx.x; t < n2; t += blockDim.x) {
        int i = (int)(t % (g.nxg - 2)) + 1, k = (int)(t / (g.nxg - 2)) + 1;
        double t2 = w0 * (double)W(i, jj, k) + w1 * (double)W(i, jj + 1, k);
        sw += t2;
        sw2 += t2 * t2;
    }
    // Vmean and UV: V(2:nxg-1, jj, 2:nzg-1), term(1:nxg-2, jj, 2:nzg-1)
    long n3 = (long)(g.nxg - 2) * (g.nzg - 2);
    for (long t = threadIdx.x; t < n3; t += blockDim.x) {
        int i = (int)(t % (g.nxg - 2)) + 2, k = (int)(t / (g.nxg - 2)) + 2;
        double v = (double)V(i, jj, k);
        double ta = w0 * (double)U(i - 1, jj, k) + w1 * (double)U(i - 1, jj + 1, k);
        double tb = w0 * (double)U(i, jj, k) + w1 * (double)U(i, jj + 1, k);
        sv += v;
        sv2 += v * v;
        suv += v * (0.5 * (ta + tb));
    }
    double r[7] = {su, sv, sw, su2, sv2, sw2, suv};
    for (int q = 0; q < 7; q++) {
        double a = bsum(r[q], sh);
        if (threadIdx.x == 0) out[7 * (jj - 1) + q] = a;
    }
}

template <typename T>
__global__ void k_stats_wall(Geo g, Fld<T> U, Fld<T> V, Fld<T> nt, double *out) {
    __shared__ double sh[32];
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    long n1 = (long)(g.nx - 2) * (g.nzg - 2);
    for (long t = threadIdx.x; t < n1; t += blockDim.x) {
        int i = (int)(t % (g.nx - 2)) + 2, k = (int)(t / (g.nx - 2)) + 2;
        s[0] += (double)U(i, 1, k);
        s[1] += (double)U(i, 2, k);
        s[2] += (double)U(i, g.nyg - 1, k);
        s[3] += (double)U(i, g.nyg, k);
    }
    long n2 = (long)(g.nxg - 2) * (g.nzg - 2);
    for (long t = threadIdx.x; t < n2; t += blockDim.x) {
        int i = (int)(t % (g.nxg - 2)) + 2, k = (int)(t / (g.nxg - 2)) + 2;
        s[4] += (double)nt(i, 1, k) + (double)nt(i, 2, k);
        s[5] += (double)nt(i, g.nyg - 1, k) + (double)nt(i, g.nyg, k);
    }
    // mass_flow.f90:37-44 and 73-80
    long n3 = (long)(g.nx - 2) * (g.nyg - 3) * (g.nzg - 2);
    for (long t = threadIdx.x; t < n3; t += blockDim.x) {
        int i = (int)(t % (g.nx - 2)) + 2;
        long r = t / (g.nx - 2);
        int j = (int)(r % (g.nyg - 3)) + 3, k = (int)(r / (g.nyg - 3)) + 2;
        s[6] += ((double)U(i, j, k) + (double)U(i, j - 1, k)) * 0.5 * (g.yg[j] - g.yg[j - 1]);
    }
    long n4 = (long)(g.nxg - 2) * (g.ny - 1) * (g.nzg - 2);
    for (long t = threadIdx.x; t < n4; t += blockDim.x) {
        int i = (int)(t % (g.nxg - 2)) + 2;
        long r = t / (g.nxg - 2);
        int j = (int)(r % (g.ny - 1)) + 2, k = (int)(r / (g.ny - 1)) + 2;
        s[7] += ((double)V(i, j, k) + (double)V(i, j - 1, k)) * 0.5 * (g.y[j] - g.y[j - 1]);
    }
    for (int q = 0; q < 8; q++) {
        double a = bsum(s[q], sh);
        if (threadIdx.x == 0) out[q] = a;
    }
}

template <typename T>
int launch_stats(cf_ctx *ctx, int b, double *d_out) {
    if (int rc = launch_nut_materialize<T>(ctx)) return rc;
    Fld<T> U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    Fld<T> nt = make_fld<T>(ctx->nut, ctx->nxg, ctx->nyg);
    k_stats_prof<T><<<ctx->ny, 256, 0, ctx->st>>>(ctx->geo, U, V, W, d_out);
    k_stats_wall<T><<<1, 1024, 0, ctx->st>>>(ctx->geo, U, V, nt, d_out + 7 * ctx->ny);
    CF_CUDA(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// output_monitor reductions (monitor.f90:28-50): per interior plane k the sums
// and maxima of U(2:nx-1, 2:nyg-1, k), V(2:nxg-1, 2:ny-1, k),
// W(2:nxg-1, 2:nyg-1, k) (k <= nz-1) and nu_t(2:nxg-1, 2:nyg-1, k); the host
// adds the planes in order.  out[8 (k-2) + q]: q = 0..3 sums, 4..7 maxima.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double bmax(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffff, v, o));
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) sh[w] = v;
    __syncthreads();
    double r = -INFINITY;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) r = fmax(r, sh[q]);
    __syncthreads();
    return r;
}

template <typename T>
__global__ void k_monitor(Geo g, Fld<T> U, Fld<T> V, Fld<T> W, Fld<T> nt, double *out) {
    __shared__ double sh[32];
    const int k = blockIdx.x + 2;
    double s[4] = {0, 0, 0, 0}, m[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
    auto scan = [&](const Fld<T> &F, int i1, int j1, int q) {
        const int ni = i1 - 1;
        const long n = (long)ni * (j1 - 1);
        for (long t = threadIdx.x; t < n; t += blockDim.x) {
            const int i = (int)(t % ni) + 2, j = (int)(t / ni) + 2;
            const double v = (double)F(i, j, k);
            s[q] += v;
            m[q] = fmax(m[q], v);
        }
    };
    scan(U, g.nx - 1, g.nyg - 1, 0);
    scan(V, g.nxg - 1, g.ny - 1, 1);
    if (k <= g.nz - 1) scan(W, g.nxg - 1, g.nyg - 1, 2);
    scan(nt, g.nxg - 1, g.nyg - 1, 3);
    for (int q = 0; q < 4; q++) {
        const double a = bsum(s[q], sh);
        const double b = bmax(m[q], sh);
        if (threadIdx.x == 0) {
            out[8 * (k - 2) + q] = a;
            out[8 * (k - 2) + 4 + q] = b;
        }
    }
}

template <typename T>
int launch_monitor(cf_ctx *ctx, int b, double *d_out) {
    if (int rc = launch_nut_materialize<T>(ctx)) return rc;
    Fld<T> U = make_fld<T>(ctx->U[b], ctx->nx, ctx->nyg);
    Fld<T> V = make_fld<T>(ctx->V[b], ctx->nxg, ctx->ny);
    Fld<T> W = make_fld<T>(ctx->W[b], ctx->nxg, ctx->nyg);
    Fld<T> nt = make_fld<T>(ctx->nut, ctx->nxg, ctx->nyg);
    k_monitor<T><<<ctx->nzg - 2, 256, 0, ctx->st>>>(ctx->geo, U, V, W, nt, d_out);
    count_launch(ctx, "k_monitor");
    CF_CUDA(cudaGetLastError());
    return 0;
}

template int launch_monitor<double>(cf_ctx *, int, double *);
template int launch_monitor<float>(cf_ctx *, int, double *);
template int launch_stats<double>(cf_ctx *, int, double *);
template int launch_stats<float>(cf_ctx *, int, double *);
