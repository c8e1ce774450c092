// mp_f32.cu -- FP32 tracer moment propagation with the scattering recomputed on the fly.
//
// For a neutral tracer the scattering probability of link l at node r is
//   n_l/rho - w_l + lambda w_l/2 = a1_l (c_l . V(r)) + lambda w_l / 2,   V = (j + f_ext)/rho
// (drop_tracers.f90:97-100 divided by rho), so every probability of a step follows from the 3
// floats of V at the node and at its neighbours.  A step then moves 40 bytes per fluid node
// (V and P_now read, P_next written, the flag word) instead of a 18-entry table; the VACF node
// sum is accumulated in FP64.
#include "common.cuh"
#include "lbgpu.h"
#include "mp.h"
#include "reduce.cuh"

namespace lbg {
namespace {

__device__ __forceinline__ void nb_offsets32(unsigned node, int lx, int ly, int lz, int (&X)[3],
                                             int (&Y)[3], int (&Z)[3])
{
    const int x = (int)(node % (unsigned)lx);
    const unsigned yz = node / (unsigned)lx;
    const int y = (int)(yz % (unsigned)ly), z = (int)(yz / (unsigned)ly);
    const int sy = lx, sz = lx * ly;
    X[0] = wrap_minus(x, lx);       X[1] = x;       X[2] = wrap_plus(x, lx);
    Y[0] = wrap_minus(y, ly) * sy;  Y[1] = y * sy;  Y[2] = wrap_plus(y, ly) * sy;
    Z[0] = wrap_minus(z, lz) * sz;  Z[1] = z * sz;  Z[2] = wrap_plus(z, lz) * sz;
}

template <int CX, int CY, int CZ>
__device__ __forceinline__ float cdot(float x, float y, float z)
{
    float s = 0.0f;
    if constexpr (CX > 0) s += x;
    if constexpr (CX < 0) s -= x;
    if constexpr (CY > 0) s += y;
    if constexpr (CY < 0) s -= y;
    if constexpr (CZ > 0) s += z;
    if constexpr (CZ < 0) s -= z;
    return s;
}

// INIT: P(t=1) and VACF(0) (module_moment_propagation.f90:112-136); else one step
// (module_moment_propagation.f90:207-253).
template <bool INIT>
__global__ void __launch_bounds__(MP_BLOCK) k_mp32(const MpArgs32 a, float bw)
{
    const volatile MpCtl *vc = a.ctl;
    if (!INIT && vc->done) return;
    const int par = INIT ? 0 : vc->parity;
    const unsigned r = blockIdx.x * MP_BLOCK + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    unsigned bad = 0;
    if (r < (unsigned)a.N) {
        const uint32_t m = __ldg(a.mask + r);
        if (m & FLUID_BIT) {
            int X[3], Y[3], Z[3];
            nb_offsets32(r, a.lx, a.ly, a.lz, X, Y, Z);
            const float vx = __ldg(a.V[0] + r), vy = __ldg(a.V[1] + r), vz = __ldg(a.V[2] + r);
            const float *__restrict__ Px = a.P[par][0];
            const float *__restrict__ Py = a.P[par][1];
            const float *__restrict__ Pz = a.P[par][2];
            float frac = 1.0f, ux = 0.0f, uy = 0.0f, uz = 0.0f;
            float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
            float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f;
            float p0 = 0.0f, p1 = 0.0f, p2 = 0.0f;
            if constexpr (!INIT) {
                p0 = Px[r];
                p1 = Py[r];
                p2 = Pz[r];
            }
            static_for<1, Q>([&](auto L) {
                constexpr int l = decltype(L)::value;
                constexpr Vel c = vel(l);
                constexpr int w = wclass(l);
                if ((m >> inv(l)) & 1u) return;  // r + c_l is solid
                const float sp = a.a1[w] * cdot<c.x, c.y, c.z>(vx, vy, vz) + a.lwh[w];
                frac -= sp;
                ux += c.x * sp;
                uy += c.y * sp;
                uz += c.z * sp;
                const unsigned rp = (unsigned)(X[c.x + 1] + Y[c.y + 1] + Z[c.z + 1]);
                const float spp =
                    a.a1[w] * cdot<-c.x, -c.y, -c.z>(__ldg(a.V[0] + rp), __ldg(a.V[1] + rp), __ldg(a.V[2] + rp)) +
                    a.lwh[w];
                if constexpr (INIT) {
                    v0 += c.x * c.x * sp;
                    v1 += c.y * c.y * sp;
                    v2 += c.z * c.z * sp;
                    n0 -= c.x * spp;
                    n1 -= c.y * spp;
                    n2 -= c.z * spp;
                } else {
                    // flux form: what arrives from r + c_l minus what leaves along l.  The
                    // probability a node keeps, 1 - sum(sp), is never formed, so its FP32
                    // rounding cannot bias the total probability step after step.
                    n0 += Px[rp] * spp - p0 * sp;
                    n1 += Py[rp] * spp - p1 * sp;
                    n2 += Pz[rp] * spp - p2 * sp;
                }
            });
            if constexpr (INIT) {
                a.P[0][0][r] = n0 * bw;
                a.P[0][1][r] = n1 * bw;
                a.P[0][2][r] = n2 * bw;
                v[0] = (double)bw * v0;
                v[1] = (double)bw * v1;
                v[2] = (double)bw * v2;
                const float fr = (a.ads && (m & INTERFACIAL_BIT)) ? frac - a.ka : frac;
                if (fr < 1.1920929e-07f) bad = LBGPU_ERR_FRACTION;
            } else {
                v[0] = (double)p0 * ux;
                v[1] = (double)p1 * uy;
                v[2] = (double)p2 * uz;
                if (!a.ads || !(m & INTERFACIAL_BIT)) {
                    n0 += p0;
                    n1 += p1;
                    n2 += p2;
                } else {
                    const float q0 = a.A[par][0][r], q1 = a.A[par][1][r], q2 = a.A[par][2][r];
                    n0 += (p0 - a.ka * p0) + q0 * a.kd;
                    n1 += (p1 - a.ka * p1) + q1 * a.kd;
                    n2 += (p2 - a.ka * p2) + q2 * a.kd;
                    a.A[par ^ 1][0][r] = q0 * a.one_minus_kd + p0 * a.ka;
                    a.A[par ^ 1][1][r] = q1 * a.one_minus_kd + p1 * a.ka;
                    a.A[par ^ 1][2][r] = q2 * a.one_minus_kd + p2 * a.ka;
                }
                __stcs(a.P[par ^ 1][0] + r, n0);
                __stcs(a.P[par ^ 1][1] + r, n1);
                __stcs(a.P[par ^ 1][2] + r, n2);
            }
        }
    }
    if constexpr (INIT) {
        __shared__ double sh[MP_BLOCK / 32];
        for (int d = 0; d < 3; ++d) {
            const double b = block_sum_fixed(v[d], sh);
            if (threadIdx.x == 0) a.partial[3 * blockIdx.x + d] = b;
        }
        if (bad) atomicOr(&a.ctl->status, bad);
    } else {
        grid_sum3(v, a.partial, &a.ctl->blocks_done,
                  [&](const double (&tot)[3]) { mp_control(a.ctl, a.hist, tot); });
    }
}

// V = (j + f_ext - rho q D E)/rho on fluid nodes (FP64, rounded once to FP32).
__global__ void __launch_bounds__(MP_BLOCK) k_mp_v(const MpArgs64 a, float *V0, float *V1, float *V2)
{
    const long long r = (long long)blockIdx.x * MP_BLOCK + threadIdx.x;
    if (r >= a.N) return;
    if (!(a.mask[r] & FLUID_BIT)) {
        V0[r] = V1[r] = V2[r] = 0.0f;
        return;
    }
    const double rho = a.rho[r];
    const double J[3] = {a.jx[r], a.jy[r], a.jz[r]};
    float *V[3] = {V0, V1, V2};
    for (int d = 0; d < 3; ++d)
        V[d][r] = (float)((J[d] + a.fext[d] - rho * a.q * a.D * a.E[d]) / rho);
}

}  // namespace

cudaError_t launch_mp_v32(const MpArgs64 &a64, float *V0, float *V1, float *V2, cudaStream_t s)
{
    k_mp_v<<<(unsigned)((a64.N + MP_BLOCK - 1) / MP_BLOCK), MP_BLOCK, 0, s>>>(a64, V0, V1, V2);
    return cudaGetLastError();
}

cudaError_t launch_mp_step_f32(const MpArgs32 &a, unsigned grid, cudaStream_t s)
{
    k_mp32<false><<<grid, MP_BLOCK, 0, s>>>(a, 0.0f);
    return cudaGetLastError();
}

cudaError_t launch_mp_init_f32(const MpArgs32 &a, float bw, unsigned grid, cudaStream_t s)
{
    k_mp32<true><<<grid, MP_BLOCK, 0, s>>>(a, bw);
    return cudaGetLastError();
}

}  // namespace lbg
