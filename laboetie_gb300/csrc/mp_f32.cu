// mp_f32.cu -- FP32 tracer moment propagation with the scattering recomputed on the fly.
//
// For a neutral tracer the scattering probability of link l at node r is
//   n_l/rho - w_l + lambda w_l/2 = a1_l (c_l . V(r)) + lambda w_l / 2,   V = (j + f_ext)/rho
// (drop_tracers.f90:97-100 divided by rho), so every probability of a step follows from V at
// the node and at its neighbours.  V and the propagated quantity P are stored as float4
// records (x, y, z, unused); the init pass also stores each fluid node's fixed (u*, D) (below).
// Boxes at least 32 x 8 wide are stepped by k_mp32_slab, which stages planes of V and P in shared
// memory (mp_slab.cuh); others by k_mp32, where a link costs two 16-byte gathers.  A step moves
// 40 algorithmic bytes per fluid node (V and P read, P written, the flag word; the code also
// reads the node's (u*, D)); the VACF node sum is formed per thread in FP32 over a few nodes and
// in FP64 across threads and blocks.  Solid neighbours hold V = 0 and P = 0 and their links are
// masked to zero, so the gathers are branch-free and can all be in flight at once.
#include <cudaTypedefs.h>

#include <cstring>

#include "common.cuh"
#include "cpasync.cuh"
#include "lbgpu.h"
#include "mp.h"
#include "mp_slab.cuh"
#include "reduce.cuh"

namespace lbg {
namespace {

// INIT: P(t=1) and VACF(0) (module_moment_propagation.f90:112-136), and the node's fixed
// aux = (u*, D); else one step (module_moment_propagation.f90:207-253) in difference form:
//   P_next(r) = P(r) + [sum_l sp_in(l) (P(r+c_l) - P(r)) + D P(r)]   (+ adsorption terms)
// which is (1 - sum sp_out) P(r) + sum_l P(r+c_l) sp_in(l) without ever forming the remaining
// fraction 1 - sum sp_out, whose FP32 rounding would otherwise bias the total probability by
// the same amount at every step: the bracket is a small correction to P(r) wherever P varies
// slowly, and D (a sum of exact FP32 link values formed in FP64) is a small net in-minus-out
// scattering.  The outgoing scatterings enter a step only through u* (the VACF) and D, both fixed
// for the run, so a step evaluates the 18 incoming ones and no outgoing one.
// The per-link operations (mp32_scatter, mp32_link) and the end of the step (mp32_finish) are
// shared with mp_slab.cuh and explicitly rounded, so both kernels give identical P.
// module_moment_propagation.f90:303-322 in FP32: phi(r') - phi(r) with the elec_slope correction
// of a link across the periodic boundary (only the first matching case of the chain).
__device__ __forceinline__ float dphi32(const MpArgs32 &a, float phi_r, float phi_p, int x, int y, int z,
                                       int xp, int yp, int zp)
{
    float d = phi_p - phi_r;
    if (x == a.lx - 1 && xp == 0) d += a.E[0] * (float)(a.lx + 1);
    else if (x == 0 && xp == a.lx - 1) d -= a.E[0] * (float)(a.lx + 1);
    else if (y == a.ly - 1 && yp == 0) d += a.E[1] * (float)(a.ly + 1);
    else if (y == 0 && yp == a.ly - 1) d -= a.E[1] * (float)(a.ly + 1);
    else if (z == a.lz - 1 && zp == 0) d += a.E[2] * (float)(a.lz + 1);
    else if (z == 0 && zp == a.lz - 1) d -= a.E[2] * (float)(a.lz + 1);
    return d;
}

// CHARGED: the scatterings carry the link's fermi factor 1/(1 + exp(z dphi)) (out of the node)
// and 1 - fermi (into it), P(t=1) the factor exp(-z dphi) and each node its Boltzmann weight
// exp(-z phi)/Pstat (module_moment_propagation.f90:97-135, 223-229, 295-327); bw is then unused.
template <bool INIT, bool CHARGED>
__global__ void __launch_bounds__(MP_BLOCK) k_mp32(const MpArgs32 a, float bw)
{
    const volatile MpCtl *vc = a.ctl;
    if (!INIT && vc->done) return;
    const int par = INIT ? 0 : vc->parity;
    const float4 *__restrict__ Pn = a.P[par];
    const float4 *__restrict__ V = a.V;
    // VACF partial of this thread: a few nodes summed in FP32, then FP64 across threads/blocks
    float vt[3] = {0.0f, 0.0f, 0.0f};
    unsigned bad = 0;
    const unsigned N = (unsigned)a.N;
    // the fluid nodes through their packed positions (every lane of a warp works), else every
    // lattice node
    const unsigned n_it = a.cpos ? a.Nf : N;
    for (unsigned i = blockIdx.x * MP_BLOCK + threadIdx.x; i < n_it; i += gridDim.x * MP_BLOCK) {
        unsigned r;
        int x, y, z;
        if (a.cpos) {
            const uint32_t c = __ldg(a.cpos + i);
            x = (int)(c & ((1u << a.xbits) - 1u));
            y = (int)((c >> a.xbits) & ((1u << a.ybits) - 1u));
            z = (int)(c >> (a.xbits + a.ybits));
            r = (unsigned)x + (unsigned)a.lx * ((unsigned)y + (unsigned)a.ly * (unsigned)z);
        } else {
            r = i;
            x = (int)(r % (unsigned)a.lx);
            const unsigned yz = r / (unsigned)a.lx;
            y = (int)(yz % (unsigned)a.ly);
            z = (int)(yz / (unsigned)a.ly);
        }
        const uint32_t m = __ldg(a.mask + r);
        if (!(m & FLUID_BIT)) continue;
        const int sy = a.lx, sz = a.lx * a.ly;
        // [c+1] = coordinate of (x + c), periodic
        const int X[3] = {wrap_minus(x, a.lx), x, wrap_plus(x, a.lx)};
        const int Y[3] = {wrap_minus(y, a.ly) * sy, y * sy, wrap_plus(y, a.ly) * sy};
        const int Z[3] = {wrap_minus(z, a.lz) * sz, z * sz, wrap_plus(z, a.lz) * sz};
        const float4 vr = __ldg(V + r);
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (!INIT) p = __ldg(Pn + r);
        float frac = 1.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
        float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
        float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f;
        double dnet = 0.0;
        // a step sums the links in mp_link_order (that of the slab step), the init in link order
        static_for<1, Q>([&](auto L) {
            constexpr int l = INIT ? decltype(L)::value : mp_link_order(decltype(L)::value);
            constexpr Vel c = vel(l);
            constexpr int w = wclass(l);
            const bool blocked = (m >> inv(l)) & 1u;  // r + c_l is solid
            const unsigned rp = (unsigned)(X[c.x + 1] + Y[c.y + 1] + Z[c.z + 1]);
            const float4 vn = __ldg(V + rp);
            float lw_out = a.lwh[w], lw_in = a.lwh[w], emd = 1.0f;
            if constexpr (CHARGED) {
                const float e = expf(a.z * dphi32(a, vr.w, vn.w, x, y, z, X[c.x + 1], Y[c.y + 1] / sy,
                                                  Z[c.z + 1] / sz));
                const float fermi = 1.0f / (1.0f + e);
                lw_out = a.lw[w] * fermi;
                lw_in = a.lw[w] * (1.0f - fermi);
                emd = blocked ? 0.0f : 1.0f / e;
            }
            const float spp = mp32_scatter(blocked, a.a1[w], mp32_cdot<-c.x, -c.y, -c.z>(vn), lw_in);
            if constexpr (INIT) {
                const float sp = mp32_scatter(blocked, a.a1[w], mp32_cdot<c.x, c.y, c.z>(vr), lw_out);
                frac -= sp;
                ux += c.x * sp;
                uy += c.y * sp;
                uz += c.z * sp;
                dnet += (double)spp - (double)sp;
                v0 += c.x * c.x * sp;
                v1 += c.y * c.y * sp;
                v2 += c.z * c.z * sp;
                const float t = CHARGED ? emd * spp : spp;
                n0 -= c.x * t;
                n1 -= c.y * t;
                n2 -= c.z * t;
            } else {
                mp32_link(spp, __ldg(Pn + rp), p, n0, n1, n2);
            }
        });
        if constexpr (INIT) {
            const float bwr = CHARGED ? expf(-(a.z * vr.w)) * a.inv_pstat : bw;
            a.P[0][r] = make_float4(n0 * bwr, n1 * bwr, n2 * bwr, 0.0f);
            a.aux[r] = make_float4(ux, uy, uz, (float)dnet);
            vt[0] += CHARGED ? v0 * bwr : v0;
            vt[1] += CHARGED ? v1 * bwr : v1;
            vt[2] += CHARGED ? v2 * bwr : v2;
            const float fr = (a.ads && (m & INTERFACIAL_BIT)) ? frac - a.ka : frac;
            if (fr < 1.1920929e-07f) bad = LBGPU_ERR_FRACTION;
        } else {
            const float4 ax = __ldg(a.aux + r);
            vt[0] += p.x * ax.x;
            vt[1] += p.y * ax.y;
            vt[2] += p.z * ax.z;
            mp32_finish(p, ax.w, n0, n1, n2);
            if (a.ads && (m & INTERFACIAL_BIT))
                a.A[par ^ 1][r] = mp32_adsorb(p, a.A[par][r], a.ka, a.kd, a.one_minus_kd, n0, n1, n2);
            __stcs(a.P[par ^ 1] + r, make_float4(n0, n1, n2, 0.0f));
        }
    }
    double v[3] = {(double)vt[0], (double)vt[1], (double)vt[2]};
    if constexpr (INIT) {
        if (!CHARGED)
            for (int d = 0; d < 3; ++d) v[d] *= (double)bw;
        block_sum3_fixed(v);
        if (threadIdx.x == 0)
            for (int d = 0; d < 3; ++d) a.partial[3 * blockIdx.x + d] = v[d];
        if (bad) atomicOr(&a.ctl->status, bad);
    } else {
        grid_sum3(v, a.partial, &a.ctl->blocks_done,
                  [&](const double (&tot)[3]) { mp_control(a.ctl, a.hist, tot); });
    }
}

// One tracer step of a box with V and P staged in shared memory (mp_slab.cuh): a block owns a
// 32 x 8 column tile and a chunk of zc planes.  With use_tma, interior tiles stage their planes
// by bulk tensor copies through the tensor maps of V and P[0], P[1] (kernel parameters).
__global__ void __launch_bounds__(MP_BLOCK, 4)
    k_mp32_slab(const MpArgs32 a, int tiles_x, int tiles_y, int zc, const __grid_constant__ CUtensorMap tmV,
                const __grid_constant__ CUtensorMap tmP0, const __grid_constant__ CUtensorMap tmP1, int use_tma)
{
    const volatile MpCtl *vc = a.ctl;
    if (vc->done) return;
    const int par = vc->parity;
    extern __shared__ float4 sm4[];
    const int nxy = tiles_x * tiles_y;
    const int tile = (int)blockIdx.x % nxy, chunk = (int)blockIdx.x / nxy;
    const int z0 = chunk * zc;
    float vt[3] = {0.0f, 0.0f, 0.0f};
    mp_slab_planes(a, par, (tile % tiles_x) * MPS_TX, (tile / tiles_x) * MPS_TY, z0, min(z0 + zc, a.lz), sm4, vt,
                   use_tma ? &tmV : nullptr, use_tma ? (par ? &tmP1 : &tmP0) : nullptr, &a.ctl->status);
    double v[3] = {(double)vt[0], (double)vt[1], (double)vt[2]};
    grid_sum3(v, a.partial, &a.ctl->blocks_done,
              [&](const double (&tot)[3]) { mp_control(a.ctl, a.hist, tot); });
}

// V = (j + f_ext - rho q D E)/rho on fluid nodes (FP64, rounded once to FP32); 0 on solid.  The
// fourth component holds the potential for a charged tracer, else the node's fluid flag (1 or 0),
// which the slab step multiplies into a link's lambda w / 2 instead of testing the link's
// bounce-back bit.
__global__ void __launch_bounds__(MP_BLOCK) k_mp_v(const MpArgs64 a, float4 *V)
{
    const long long r = (long long)blockIdx.x * MP_BLOCK + threadIdx.x;
    if (r >= a.N) return;
    const bool fluid = a.mask[r] & FLUID_BIT;
    const float w = a.phi ? (float)a.phi[r] : (fluid ? 1.0f : 0.0f);
    if (!fluid) {
        V[r] = make_float4(0.f, 0.f, 0.f, w);
        return;
    }
    const double rho = a.rho[r];
    const double J[3] = {a.jx[r], a.jy[r], a.jz[r]};
    float o[3];
    for (int d = 0; d < 3; ++d) o[d] = (float)((J[d] + a.fext[d] - rho * a.q * a.D * a.E[d]) / rho);
    V[r] = make_float4(o[0], o[1], o[2], w);
}

}  // namespace

cudaError_t launch_mp_v32(const MpArgs64 &a64, float4 *V, cudaStream_t s)
{
    k_mp_v<<<(unsigned)((a64.N + MP_BLOCK - 1) / MP_BLOCK), MP_BLOCK, 0, s>>>(a64, V);
    return cudaGetLastError();
}

bool mp32_tensor_map(CUtensorMap *tm, const float4 *field, int lx, int ly, int lz)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            return false;
        }
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    // the float4 field as a 4-D FP32 tensor (component, x, y, z); box = one plane of a tile with
    // its halo (4 x 34 x 10 x 1), landing as the ring plane's SHX x SHY float4 records
    const cuuint64_t dims[4] = {4, (cuuint64_t)lx, (cuuint64_t)ly, (cuuint64_t)lz};
    const cuuint64_t strides[3] = {16, 16ull * (cuuint64_t)lx, 16ull * (cuuint64_t)lx * (cuuint64_t)ly};
    const cuuint32_t box[4] = {4, (cuuint32_t)SHX, (cuuint32_t)SHY, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    return encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float4 *>(field), dims, strides, box,
                  estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

unsigned mp32_slab_resident()
{
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaFuncSetAttribute(k_mp32_slab, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MPS_SMEM) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mp32_slab, MP_BLOCK, MPS_SMEM) != cudaSuccess) {
        cudaGetLastError();
        return 0u;
    }
    return (unsigned)(sms * per_sm);
}

cudaError_t launch_mp_step_f32(const MpArgs32 &a, unsigned grid, const CUtensorMap *tm, cudaStream_t s)
{
    int zc = 0;
    const unsigned sg = a.slab && !a.charged ? mp32_slab_grid(a.lx, a.ly, a.lz, a.slab_resident, &zc) : 0u;
    if (sg) {
        const int tx = (a.lx + MPS_TX - 1) / MPS_TX, ty = (a.ly + MPS_TY - 1) / MPS_TY;
        CUtensorMap none;
        std::memset(&none, 0, sizeof(none));
        k_mp32_slab<<<sg, MP_BLOCK, MPS_SMEM, s>>>(a, tx, ty, zc, tm ? tm[0] : none, tm ? tm[1] : none,
                                                   tm ? tm[2] : none, tm ? 1 : 0);
    } else {
        if (a.charged) k_mp32<false, true><<<grid, MP_BLOCK, 0, s>>>(a, 0.0f);
        else k_mp32<false, false><<<grid, MP_BLOCK, 0, s>>>(a, 0.0f);
    }
    return cudaGetLastError();
}

cudaError_t launch_mp_init_f32(const MpArgs32 &a, float bw, unsigned grid, cudaStream_t s)
{
    if (a.charged) k_mp32<true, true><<<grid, MP_BLOCK, 0, s>>>(a, bw);
    else k_mp32<true, false><<<grid, MP_BLOCK, 0, s>>>(a, bw);
    return cudaGetLastError();
}

}  // namespace lbg
