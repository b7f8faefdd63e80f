// Divergence check on caller-owned device arrays that allocates no device
// memory (cf_check_divergence_noalloc in channel_gpu.h).
//
// Who needs it: callers that must not allocate device memory while they run,
// e.g. a solver that hands all device memory to its own pool at start-up and
// runs under a fixed memory cap, or a driver that cannot afford the implicit
// device synchronisation a cudaMalloc/cudaFree may cause in the middle of its
// stream work.  Such callers own U, V, W and the grid on the device but cannot
// create a cf_ctx (cf_create allocates).  This entry point needs no context:
// its only scratch is the file-scope __device__ array below, whose address is
// looked up once per device.
//
// Same arithmetic as check_divergence (projection.f90:234-256) and as the
// kernel behind cf_check_divergence: per interior cell
//   div = (U(i)-U(i-1))/(x(i)-x(i-1)) + (V(j)-V(j-1))/(y(j)-y(j-1))
//       + (W(k)-W(k-1))/(z(k)-z(k-1))
// and the results max(0, max div) (the reference's Max starting from 0) and
// max |div|; a NaN divergence in any cell makes both results NaN.  The
// reduction is two-stage and deterministic: one block per interior z plane
// writes that plane's two maxima to the scratch, then one block reduces the
// planes.
#include <mutex>

#include "cf_internal.cuh"

// One (max div, max |div|) pair per interior z plane: 2 x 4096 doubles = 64 KiB.
static __device__ __align__(256) double g_div_planes[2 * CF_NOALLOC_MAX_PLANES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double *g_planes_ptr[kMaxDevices] = {};  // device address of g_div_planes, per device

// max that keeps a NaN (fmax would drop it)
__device__ __forceinline__ double nan_max(double a, double b) {
    return (isnan(a) || isnan(b)) ? __longlong_as_double(0x7FF8000000000000LL) : fmax(a, b);
}

__device__ __forceinline__ void block_max2(double &d, double &a, double *sh) {
    for (int o = 16; o > 0; o >>= 1) {
        d = nan_max(d, __shfl_down_sync(0xffffffffu, d, o));
        a = nan_max(a, __shfl_down_sync(0xffffffffu, a, o));
    }
    const int t = threadIdx.x + threadIdx.y * blockDim.x, nw = (blockDim.x * blockDim.y) >> 5;
    if ((t & 31) == 0) {
        sh[2 * (t >> 5)] = d;
        sh[2 * (t >> 5) + 1] = a;
    }
    __syncthreads();
    if (t < 32) {
        d = t < nw ? sh[2 * t] : 0.0;
        a = t < nw ? sh[2 * t + 1] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            d = nan_max(d, __shfl_down_sync(0xffffffffu, d, o));
            a = nan_max(a, __shfl_down_sync(0xffffffffu, a, o));
        }
    }
}

// Block b handles the interior plane k = b + 2 (1-based); every interior cell
// i = 2..nxg-1, j = 2..nyg-1 of it.  Arrays are 1-based Fortran order:
// U(nx, nyg, nzg), V(nxg, ny, nzg), W(nxg, nyg, nz), x(nx), y(ny), z(nz).
__global__ void __launch_bounds__(256) k_div_planes(int nx, int ny, int nz, const double *__restrict__ U,
                                                    const double *__restrict__ V, const double *__restrict__ W,
                                                    const double *__restrict__ x, const double *__restrict__ y,
                                                    const double *__restrict__ z, double *__restrict__ planes) {
    __shared__ double sh[16];
    const int nxg = nx + 1, nyg = ny + 1;
    const int k = blockIdx.x + 2;
    const double dz = z[k - 1] - z[k - 2];
    const size_t pu = (size_t)nx * nyg, pv = (size_t)nxg * ny, pw = (size_t)nxg * nyg;
    const double *Uk = U + pu * (k - 1), *Vk = V + pv * (k - 1), *Wk = W + pw * (k - 1), *Wm = W + pw * (k - 2);
    double d = 0.0, a = 0.0;
    for (int j = 2 + threadIdx.y; j <= nyg - 1; j += blockDim.y) {
        const double dy = y[j - 1] - y[j - 2];
        for (int i = 2 + threadIdx.x; i <= nxg - 1; i += blockDim.x) {
            const double v = (Uk[(i - 1) + (size_t)nx * (j - 1)] - Uk[(i - 2) + (size_t)nx * (j - 1)]) / (x[i - 1] - x[i - 2]) +
                             (Vk[(i - 1) + (size_t)nxg * (j - 1)] - Vk[(i - 1) + (size_t)nxg * (j - 2)]) / dy +
                             (Wk[(i - 1) + (size_t)nxg * (j - 1)] - Wm[(i - 1) + (size_t)nxg * (j - 1)]) / dz;
            d = nan_max(d, v);
            a = nan_max(a, fabs(v));
        }
    }
    block_max2(d, a, sh);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        planes[2 * blockIdx.x] = d;
        planes[2 * blockIdx.x + 1] = a;
    }
}

__global__ void __launch_bounds__(256) k_div_planes_final(int nplanes, const double *__restrict__ planes,
                                                          double *__restrict__ out) {
    __shared__ double sh[16];
    double d = 0.0, a = 0.0;
    for (int p = threadIdx.x; p < nplanes; p += blockDim.x) {
        d = nan_max(d, planes[2 * p]);
        a = nan_max(a, planes[2 * p + 1]);
    }
    block_max2(d, a, sh);
    if (threadIdx.x == 0) {
        out[0] = d;
        out[1] = a;
    }
}

bool device_pointer(const void *p, int dev) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeManaged) return true;
    return at.type == cudaMemoryTypeDevice && at.device == dev;
}
}  // namespace

extern "C" int cf_check_divergence_noalloc(int nx, int ny, int nz, const double *U, const double *V,
                                           const double *W, const double *x, const double *y, const double *z,
                                           double *out, void *stream) {
    cf_ctx *ctx = nullptr;  // errors go to cf_last_error(NULL)
    if (nx < 2 || ny < 2 || nz < 2)
        return cf_fail(ctx, CF_ERR_INVALID, "cf_check_divergence_noalloc: nx, ny, nz must be >= 2");
    const int nplanes = nz - 1;  // interior planes k = 2 .. nzg-1
    if (nplanes > CF_NOALLOC_MAX_PLANES)
        return cf_fail(ctx, CF_ERR_INVALID,
                       "cf_check_divergence_noalloc: nz - 1 = " + std::to_string(nplanes) +
                           " interior z planes exceed the static scratch of " +
                           std::to_string(CF_NOALLOC_MAX_PLANES) + " planes");
    if (!U || !V || !W || !x || !y || !z || !out)
        return cf_fail(ctx, CF_ERR_INVALID, "cf_check_divergence_noalloc: null argument");
    int dev = 0;
    CF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return cf_fail(ctx, CF_ERR_UNSUPPORTED, "cf_check_divergence_noalloc: device index >= 64");
    const void *ptrs[7] = {U, V, W, x, y, z, out};
    for (const void *p : ptrs)
        if (!device_pointer(p, dev))
            return cf_fail(ctx, CF_ERR_INVALID,
                           "cf_check_divergence_noalloc: every array must be device (or managed) memory "
                           "of the current device");
    double *planes;
    {
        // One-time setup per device, with that device current: the scratch address.
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_planes_ptr[dev]) {
            void *p = nullptr;
            CF_CUDA(cudaGetSymbolAddress(&p, g_div_planes));
            g_planes_ptr[dev] = static_cast<double *>(p);
        }
        planes = g_planes_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_div_planes<<<nplanes, dim3(64, 4), 0, st>>>(nx, ny, nz, U, V, W, x, y, z, planes);
    CF_CUDA(cudaGetLastError());
    k_div_planes_final<<<1, 256, 0, st>>>(nplanes, planes, out);
    CF_CUDA(cudaGetLastError());
    return CF_OK;
}
