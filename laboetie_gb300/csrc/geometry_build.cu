// geometry_build.cu -- the reference's geometry builders on the device (module_geometry.f90,
// selected by geometryLabel in supercell_definition.f90:52-80): one thread per node writes
// node%nature (0 fluid, 1 solid).  Compiled without fused multiply-add: every distance is
// gfortran's NORM2 (scaled sum of squares, separately rounded operations), so nodes at exactly
// the threshold distance fall on the same side as in the reference.  The box-level constants
// (radii, centres, thresholds) are evaluated on the host in the reference's operation order and
// precision (default-REAL literals and conversions in single precision).  Labels 0 (geom.in)
// and 11 (geom.pbm) read files and stay with the host.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "ctx.h"
#include "lbgpu.h"

namespace lbg {
namespace {

constexpr int BLOCK = 256;

struct GeomArgs {
    int label, lx, ly, lz;
    double c[8];   // per-label constants (see geom_constants)
};

// gfortran's inline NORM2: scale starts at 1; each non-zero component either rescales the sum
// (when larger than the scale) or adds its square relative to the scale.
template <int NC>
__device__ __forceinline__ double norm2_dev(const double (&v)[NC])
{
    double scale = 1.0, ssq = 0.0;
#pragma unroll
    for (int q = 0; q < NC; ++q) {
        if (v[q] != 0.0) {
            const double ax = fabs(v[q]);
            if (scale < ax) {
                const double t = scale / ax;
                ssq = 1.0 + ssq * t * t;
                scale = ax;
            } else {
                const double t = ax / scale;
                ssq = ssq + t * t;
            }
        }
    }
    return scale * sqrt(ssq);
}

__device__ __forceinline__ double dist2(double a, double b)
{
    const double v[2] = {a, b};
    return norm2_dev(v);
}

__device__ __forceinline__ double dist3(double a, double b, double c)
{
    const double v[3] = {a, b, c};
    return norm2_dev(v);
}

// node%nature of the 1-based node (i, j, k)
__device__ int8_t nature_of(const GeomArgs &g, int i, int j, int k)
{
    const int lx = g.lx, ly = g.ly, lz = g.lz;
    const double x = (double)i, y = (double)j, z = (double)k;
    switch (g.label) {
    case 1:   // module_geometry.f90:158-166
        return (k == 1 || k == lz) ? 1 : 0;
    case 2:   // :253-277, c = {origin x, origin y, radius}
        return dist2(x - g.c[0], y - g.c[1]) >= g.c[2] ? 1 : 0;
    case 3: { // :206-245, c = {threshold, centre}: spheres at the 8 corners and the centre
        const double thr = g.c[0];
        const double cx[2] = {1.0, (double)lx}, cy[2] = {1.0, (double)ly}, cz[2] = {1.0, (double)lz};
        bool in = dist3(x - g.c[1], y - g.c[2], z - g.c[3]) <= thr;
        for (int q = 0; q < 8; ++q)
            in = in || dist3(x - cx[q & 1], y - cy[(q >> 1) & 1], z - cz[q >> 2]) <= thr;
        return in ? 1 : 0;
    }
    case 4:   // :336-378, c = {origin x, origin y, radius}
        return dist2(x - g.c[0], y - g.c[1]) > g.c[2] ? 1 : 0;
    case 5: { // :122-153, c = {a, b, midly, 2 pi}
        const int midly = (int)g.c[2];
        const double yi = g.c[0] * sin(g.c[3] * (double)(i - 1) / (double)lx) + g.c[1] + g.c[2];
        const long long ninty = llround(yi);          // NINT: half away from zero
        const int jj = j >= midly ? j : 2 * midly - j;   // rows below the middle mirror those above
        return (long long)jj < ninty ? 0 : 1;
    }
    case 6: { // :96-119
        if (j == 1 || j == ly) return 1;
        const int q = (ly - 2) / 4;
        return (i > lx / 2 && ((j >= 2 && j <= 1 + q) || (j >= ly - q && j <= ly - 1))) ? 1 : 0;
    }
    case 7: { // :52-89, c = {lw_o_lx * lx, a, R, r0 y, r0 z}
        const double d = dist2((double)(float)j - g.c[3], (double)(float)k - g.c[4]);
        const bool fluid = x > g.c[0] ? d < g.c[1] : d < g.c[2];
        return fluid ? 0 : 1;
    }
    case 8:   // :173-198, c = {origin, radius}
        return dist3(x - g.c[0], y - g.c[0], z - g.c[0]) >= g.c[1] ? 1 : 0;
    case 9:   // :287-331, c = {origin, radius}
        return dist3(x - g.c[0], y - g.c[0], z - g.c[0]) > g.c[1] ? 1 : 0;
    case 10: { // :11-49, c = {midx, midy, radius}
        if (k == 1 || k == lz) return 1;
        const double cx[4] = {1.0, (double)lx, g.c[0], g.c[0]}, cy[4] = {g.c[1], g.c[1], 1.0, (double)ly};
        for (int q = 0; q < 4; ++q)
            if (dist2(x - cx[q], y - cy[q]) <= g.c[2]) return 1;
        return 0;
    }
    default:  // -1: no solid node
        return 0;
    }
}

__global__ void __launch_bounds__(BLOCK) k_geometry(const GeomArgs g, int8_t *__restrict__ nature,
                                                     unsigned long long *__restrict__ nfluid)
{
    const long long N = (long long)g.lx * g.ly * g.lz;
    const long long node = (long long)blockIdx.x * BLOCK + threadIdx.x;
    int8_t v = 1;
    if (node < N) {
        const int i = (int)(node % g.lx) + 1;
        const long long jk = node / g.lx;
        const int j = (int)(jk % g.ly) + 1, k = (int)(jk / g.ly) + 1;
        v = nature_of(g, i, j, k);
        nature[node] = v;
    }
    const unsigned fl = __ballot_sync(0xffffffffu, v == 0);
    if ((threadIdx.x & 31) == 0 && fl) atomicAdd(nfluid, (unsigned long long)__popc(fl));
}

// The reference's checks of the box for the label (its STOP messages) and the box constants in
// its operation order.  Returns an empty string when the box is accepted.
std::string geom_constants(int label, int lx, int ly, int lz, const double *params, GeomArgs &g)
{
    g.label = label;
    g.lx = lx;
    g.ly = ly;
    g.lz = lz;
    for (double &v : g.c) v = 0.0;
    switch (label) {
    case -1:
    case 1:
    case 6:
        return "";
    case 2:
        if (lx != ly) return "wall=2 is for cylinders, which should have same lx and ly";
        if (lx < 3) return "the diameter of the cylinder (lx) should be greater than 3";
        g.c[0] = (double)(lx + 1) / 2.0;
        g.c[1] = (double)(ly + 1) / 2.0;
        g.c[2] = (double)(lx - 1) / 2.0;
        return "";
    case 3:
        if (lx != ly || lx != lz)
            return "with wall = 3, i.e. cfc cell, the supercell should be cubic with lx=ly=lz";
        g.c[0] = (double)(lx - 1) * std::sqrt(3.0) / 4.0;
        g.c[1] = (double)(float)(lx + 1) / 2.0;   // real([lx+1,ly+1,lz+1])/2._dp
        g.c[2] = (double)(float)(ly + 1) / 2.0;
        g.c[3] = (double)(float)(lz + 1) / 2.0;
        return "";
    case 4: {
        if (lx != ly) return "wall=4 should have same lx and ly";
        if (lx % 2 == 0) return "lx should be odd";
        g.c[0] = (double)(lx + 1) / 2.0;
        g.c[1] = (double)(ly + 1) / 2.0;
        // norm2([1, (lx+1)/2] - rorigin): the second component is 0 (lx == ly, odd), and NORM2
        // of one non-zero component is its magnitude
        g.c[2] = std::fabs(1.0 - g.c[0]);
        return "";
    }
    case 5: {
        if (ly % 2 == 0) return "ly should be odd";
        const int midly = (ly + 1) / 2;
        const double b = (double)((float)(2.0f / 3.0f) * (float)midly);   // 2./3.*midly, REAL
        const double a = (double)midly - b - 1.0;
        if (a <= 0.0 || b <= 0.0) return "pb in def geometry function";
        g.c[0] = a;
        g.c[1] = b;
        g.c[2] = (double)midly;
        g.c[3] = 2.0 * 3.141592653589793;   // 2._dp*acos(-1.0_dp)
        return "";
    }
    case 7: {
        if (ly != lz) return "ly should be equal to lz cause it is a tube";
        if (!params) return "tube.in cannot be read";
        const double R = (double)((float)(ly - 1) / 2.0f);   // real(ly-1)/2.0, REAL
        g.c[0] = params[0] * (double)lx;                      // lw_o_lx*lx
        g.c[1] = params[1] * R;                               // a = a_o_R*R
        g.c[2] = R;
        g.c[3] = (double)((float)(ly + 1) / 2.0f);
        g.c[4] = (double)((float)(lz + 1) / 2.0f);
        return "";
    }
    case 8:
        if (lx != ly || lx != lz) return "wall=8 for a spherical cavity so lx=ly=lz. check input file.";
        if (lx < 3) return "the diameter of the cylinder (lx) should be greater than 3";
        g.c[0] = (double)(lx + 1) / 2.0;
        g.c[1] = (double)(lx - 1) / 2.0;
        return "";
    case 9: {
        if (lx != ly || lx != lz) return "wall=9 should have same lx, ly and lz";
        if (lx % 2 == 0) return "lx should be odd";
        g.c[0] = (double)(lx + 1) / 2.0;
        // norm2([1, (ly+1)/2, (lz+1)/2] - rorigin) = |1 - origin| (the other components are 0)
        g.c[1] = std::fabs(1.0 - g.c[0]);
        return "";
    }
    case 10: {
        const float s3 = std::sqrt(3.0f);
        if (std::fabs((float)ly / (float)lx - s3) / s3 >= 0.05f)
            return "STOP. ly shoud be lx *sqrt(3). Ly should be " + std::to_string(lx * std::sqrt(3.0f));
        if (lz < 3) return "Lz should be greater than 2 because there are two walls. STOP";
        g.c[0] = (double)(lx + 1) / 2.0;
        g.c[1] = (double)(ly + 1) / 2.0;
        g.c[2] = 0.2 * (double)lx;
        return "";
    }
    case 0:
    case 11:
        return "geometryLabel " + std::to_string(label) +
               " reads geom." + (label == 0 ? "in" : "pbm") + " on the host: pass its nature to lbgpu_create";
    default:
        return "supercell%geometry%label tag in input file is invalid";
    }
}

}  // namespace

// Builds the box on the device into d_nature (N bytes); *nfluid = fluid node count.
int geometry_build(int label, int lx, int ly, int lz, const double *params, int8_t *d_nature,
                   long long *nfluid, cudaStream_t s, std::string &err)
{
    GeomArgs g;
    err = geom_constants(label, lx, ly, lz, params, g);
    if (!err.empty()) return LBGPU_ERR_INVALID;
    const long long N = (long long)lx * ly * lz;
    unsigned long long *d_cnt = nullptr;
    cudaError_t e = cudaMallocAsync(&d_cnt, sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        k_geometry<<<(unsigned)((N + BLOCK - 1) / BLOCK), BLOCK, 0, s>>>(g, d_nature, d_cnt);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_cnt, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (d_cnt) cudaFreeAsync(d_cnt, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        err = std::string("lbgpu_geometry: ") + cudaGetErrorString(e);
        return LBGPU_ERR_CUDA;
    }
    *nfluid = (long long)h;
    if (h == 0) {   // supercell_definition.f90:92-94
        err = "All nodes are solid: no fluid, no fluid dynamics!";
        return LBGPU_ERR_INVALID;
    }
    return LBGPU_OK;
}

// Host-side check of a label and box without a GPU (the reference's STOP conditions).
int geometry_check(int label, int lx, int ly, int lz, const double *params, std::string &err)
{
    GeomArgs g;
    err = geom_constants(label, lx, ly, lz, params, g);
    return err.empty() ? LBGPU_OK : LBGPU_ERR_INVALID;
}

}  // namespace lbg
