// noalloc_moments.cu -- the moments step of the flow loop on caller-owned device arrays,
// without any device allocation.
//
// Who needs this.  Some callers cannot let a library call cudaMalloc: a host that already
// keeps its populations on the GPU (allocated by its own runtime, a pool it must not grow, or
// memory it manages explicitly) and only wants density, flux and the convergence measure of
// them; code running where allocating is forbidden or too slow (inside a tight time loop with
// a fixed memory budget).  lbgpu_moments needs a context, which owns device buffers; this entry
// point needs none.  The caller passes every input and output as a device pointer; the only
// other memory used is the fixed reduction scratch below.
//
// Scratch.  One file-scope device array holds one partial result per thread block plus the
// final result: NA_MAX_BLOCKS blocks of NA_BLOCK threads, i.e. at most 16,777,216 nodes (256^3)
// per call; larger boxes are rejected.  The array is about 1 MiB and lives on every GPU that
// loads the library until the process exits.  Every call overwrites the partials of the blocks
// it launches before the final kernel reads them, so nothing carries over from a previous call
// and nothing has to be cleared.  All calls share the one array: two calls whose kernels
// overlap on the GPU (different streams, different host threads) race on it and must be
// serialised by the caller.
//
// The host side needs the device address of the array.  The first call on each device looks
// it up (cudaGetSymbolAddress, with that device current) and caches it.  Every call ends by
// copying l2err back and waiting for its stream, so no call can be captured into a CUDA graph.
//
// Results match lbgpu_moments bit for bit, including on non-finite input: l2err is a maximum
// over IEEE bit patterns (a NaN difference gives a NaN l2err), and a NaN or infinite population
// is reported as LBGPU_ERR_NONFINITE, a negative one as LBGPU_ERR_NEGATIVE_POPULATION (the
// outputs are written either way).
#include <cuda_runtime.h>

#include <cfloat>
#include <mutex>
#include <string>

#include "common.cuh"
#include "ctx.h"
#include "lbgpu.h"

namespace {

constexpr int NA_BLOCK = 256;
constexpr unsigned NA_MAX_BLOCKS = 65536;
constexpr long long NA_MAX_NODES = (long long)NA_MAX_BLOCKS * NA_BLOCK;
constexpr int NA_MAX_DEVICES = 64;

struct __align__(16) NaPartial {
    double max_dj;    // max over the block's nodes of |j - j_old| (all three components; NaN wins)
    unsigned status;  // lbgpu_status bits raised by the block
    unsigned pad;
};

// [0, NA_MAX_BLOCKS): per-block partials; [NA_MAX_BLOCKS]: the reduced result of the call.
static __device__ __align__(256) NaPartial g_na_scratch[NA_MAX_BLOCKS + 1];

std::mutex g_na_mutex;
NaPartial *g_na_addr[NA_MAX_DEVICES] = {};

// Density, flux and the n<0 test of equilibration.f90:248,254,293-300 and the per-node part
// of l2err (339-343), in the reference's order: density = SUM(n,4) from l = 1 upward;
// j = f_ext/2 + sum_l n_l c_l with the c = 0 terms left out and c = -1 as a subtraction.
__global__ void __launch_bounds__(NA_BLOCK)
k_na_moments(const double *__restrict__ n, const double *__restrict__ fx,
             const double *__restrict__ fy, const double *__restrict__ fz, double *rho,
             double *jx, double *jy, double *jz, long long N, NaPartial *part)
{
    const long long node = (long long)blockIdx.x * NA_BLOCK + threadIdx.x;
    double err = 0.0;
    unsigned bad = 0;
    if (node < N) {
        double f[lbg::Q];
#pragma unroll
        for (int l = 0; l < lbg::Q; ++l) {
            f[l] = n[(long long)l * N + node];
            if (f[l] < 0.0) bad |= LBGPU_ERR_NEGATIVE_POPULATION;
            if (!(fabs(f[l]) <= DBL_MAX)) bad |= LBGPU_ERR_NONFINITE;
        }
        double r = f[0];
#pragma unroll
        for (int l = 1; l < lbg::Q; ++l) r = r + f[l];
        double X = fx[node] / 2.0, Y = fy[node] / 2.0, Z = fz[node] / 2.0;
        lbg::static_for<0, lbg::Q>([&](auto L) {
            constexpr int l = decltype(L)::value;
            constexpr lbg::Vel c = lbg::vel(l);
            if constexpr (c.x > 0) X = X + f[l];
            if constexpr (c.x < 0) X = X - f[l];
            if constexpr (c.y > 0) Y = Y + f[l];
            if constexpr (c.y < 0) Y = Y - f[l];
            if constexpr (c.z > 0) Z = Z + f[l];
            if constexpr (c.z < 0) Z = Z - f[l];
        });
        err = lbg::max_nonneg(lbg::max_nonneg(fabs(X - jx[node]), fabs(Y - jy[node])), fabs(Z - jz[node]));
        rho[node] = r;
        jx[node] = X;
        jy[node] = Y;
        jz[node] = Z;
    }
    // block max / or, written to this block's partial (every launched block writes its own)
    __shared__ double se[NA_BLOCK / 32];
    __shared__ unsigned sb[NA_BLOCK / 32];
    for (int o = 16; o > 0; o >>= 1) {
        err = lbg::max_nonneg(err, __shfl_xor_sync(0xffffffffu, err, o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        se[wid] = err;
        sb[wid] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double e = se[0];
        unsigned b = sb[0];
        for (int w = 1; w < NA_BLOCK / 32; ++w) {
            e = lbg::max_nonneg(e, se[w]);
            b |= sb[w];
        }
        part[blockIdx.x].max_dj = e;
        part[blockIdx.x].status = b;
    }
}

// One block: max / or over the partials of the nb blocks of this call -> part[NA_MAX_BLOCKS].
__global__ void __launch_bounds__(NA_BLOCK) k_na_reduce(NaPartial *part, unsigned nb)
{
    double e = 0.0;
    unsigned b = 0;
    for (unsigned i = threadIdx.x; i < nb; i += NA_BLOCK) {
        e = lbg::max_nonneg(e, part[i].max_dj);
        b |= part[i].status;
    }
    __shared__ double se[NA_BLOCK];
    __shared__ unsigned sb[NA_BLOCK];
    se[threadIdx.x] = e;
    sb[threadIdx.x] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int t = 1; t < NA_BLOCK; ++t) {
            e = lbg::max_nonneg(e, se[t]);
            b |= sb[t];
        }
        part[NA_MAX_BLOCKS].max_dj = e;
        part[NA_MAX_BLOCKS].status = b;
    }
}

// Device address of the scratch on the current device, looked up once per device.
int scratch_on_current_device(NaPartial **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return lbg::ctx_fail(nullptr, LBGPU_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= NA_MAX_DEVICES)
        return lbg::ctx_fail(nullptr, LBGPU_ERR_INVALID, "lbgpu_moments_noalloc: device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess || !p)
            return lbg::ctx_fail(nullptr, LBGPU_ERR_CUDA,
                                 std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_na_addr[dev] = static_cast<NaPartial *>(p);
    }
    *out = g_na_addr[dev];
    return LBGPU_OK;
}

}  // namespace

extern "C" int lbgpu_moments_noalloc(int lx, int ly, int lz, const double *d_n,
                                     const double *d_fx, const double *d_fy, const double *d_fz,
                                     double *d_density, double *d_jx, double *d_jy, double *d_jz,
                                     double *l2err, void *stream)
{
    if (!d_n || !d_fx || !d_fy || !d_fz || !d_density || !d_jx || !d_jy || !d_jz)
        return lbg::ctx_fail(nullptr, LBGPU_ERR_INVALID, "lbgpu_moments_noalloc: null device pointer");
    if (lx <= 0 || ly <= 0 || lz <= 0)
        return lbg::ctx_fail(nullptr, LBGPU_ERR_INVALID, "lbgpu_moments_noalloc: lx, ly, lz must be > 0");
    const long long N = (long long)lx * ly * lz;
    if (N > NA_MAX_NODES)
        return lbg::ctx_fail(nullptr, LBGPU_ERR_INVALID,
                             "lbgpu_moments_noalloc: " + std::to_string(N) +
                                 " nodes exceed the fixed scratch, which holds at most " +
                                 std::to_string(NA_MAX_NODES) + " nodes (256^3) per call");
    NaPartial *part = nullptr;
    int rc = scratch_on_current_device(&part);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned nb = (unsigned)((N + NA_BLOCK - 1) / NA_BLOCK);
    k_na_moments<<<nb, NA_BLOCK, 0, s>>>(d_n, d_fx, d_fy, d_fz, d_density, d_jx, d_jy, d_jz, N, part);
    k_na_reduce<<<1, NA_BLOCK, 0, s>>>(part, nb);
    cudaError_t e = cudaGetLastError();
    NaPartial res{};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&res, part + NA_MAX_BLOCKS, sizeof(res), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return lbg::ctx_fail(nullptr, LBGPU_ERR_CUDA, std::string("lbgpu_moments_noalloc: ") + cudaGetErrorString(e));
    if (l2err) *l2err = res.max_dj;
    return lbg::moments_status(nullptr, res.status);
}
