// geometry.cu -- node classification on the device (integer work, bit-exact by construction).
//
// For every node the flag word holds, for each velocity l = 1..18, whether the pull source
// node - c_l has a different nature than the node (halfway bounce-back on that link), plus the
// fluid bit and the interfacial bit.  A node is interfacial iff one of its 18 periodic
// neighbours has a different nature (supercell_definition.f90:115-147); the set of nodes
// node - c_l over all l equals the set node + c_l, so that is "any bounce-back bit set".
#include "common.cuh"
#include "flow.h"

namespace lbg {
namespace {

constexpr int BLOCK = 256;

__global__ void __launch_bounds__(BLOCK)
k_node_flags(const int8_t *__restrict__ nature, uint32_t *__restrict__ mask, int lx, int ly,
             int lz)
{
    const long long N = (long long)lx * ly * lz;
    const long long node = (long long)blockIdx.x * BLOCK + threadIdx.x;
    if (node >= N) return;
    const unsigned nd = (unsigned)node;
    const int x = (int)(nd % (unsigned)lx);
    const unsigned yz = nd / (unsigned)lx;
    const int y = (int)(yz % (unsigned)ly), z = (int)(yz / (unsigned)ly);
    const int8_t me = nature[node];
    uint32_t m = 0;
    static_for<1, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel c = vel(l);
        const int sx = c.x == 1 ? wrap_minus(x, lx) : (c.x == -1 ? wrap_plus(x, lx) : x);
        const int sy = c.y == 1 ? wrap_minus(y, ly) : (c.y == -1 ? wrap_plus(y, ly) : y);
        const int sz = c.z == 1 ? wrap_minus(z, lz) : (c.z == -1 ? wrap_plus(z, lz) : z);
        const long long s = sx + (long long)lx * (sy + (long long)ly * sz);
        if (nature[s] != me) m |= 1u << l;
    });
    if (me == 0) m |= FLUID_BIT;
    if (m & BB_BITS) m |= INTERFACIAL_BIT;
    mask[node] = m;
}

// counts[0..3] += fluid, solid, fluid&interfacial, solid&interfacial
__global__ void __launch_bounds__(BLOCK)
k_count_nodes(const uint32_t *__restrict__ mask, long long N, unsigned long long *counts)
{
    unsigned long long c[4] = {0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < N;
         i += (long long)gridDim.x * BLOCK) {
        const uint32_t m = mask[i];
        const bool f = m & FLUID_BIT, it = m & INTERFACIAL_BIT;
        c[0] += f;
        c[1] += !f;
        c[2] += f && it;
        c[3] += !f && it;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        unsigned long long v = c[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&counts[q], v);
    }
}

}  // namespace

cudaError_t launch_node_flags(const int8_t *nature, uint32_t *mask, int lx, int ly, int lz,
                              cudaStream_t s)
{
    const long long N = (long long)lx * ly * lz;
    k_node_flags<<<(unsigned)((N + BLOCK - 1) / BLOCK), BLOCK, 0, s>>>(nature, mask, lx, ly, lz);
    return cudaGetLastError();
}

cudaError_t launch_count_nodes(const uint32_t *mask, long long N, unsigned long long *counts,
                               cudaStream_t s)
{
    long long g = (N + BLOCK - 1) / BLOCK;
    if (g > 1216) g = 1216;
    if (g < 1) g = 1;
    k_count_nodes<<<(unsigned)g, BLOCK, 0, s>>>(mask, N, counts);
    return cudaGetLastError();
}

}  // namespace lbg
