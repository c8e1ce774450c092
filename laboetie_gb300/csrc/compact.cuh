// compact.cuh -- the in-place AA layout over fluid nodes only.
//
// A box's fluid nodes are numbered in lattice order (compact index i); populations live at
// g[l*Nf + i].  Per node: cpos[i] = x | y << xbits | z << (xbits + ybits) (packed position) and
// cmask[i] = its flag word.  Per lattice row (y, z) and 32-node word w: rowtab[row*nw + w] =
// {fluid bitmask of the word, compact index of the word's first fluid node}.  The helpers are
// templated on an argument struct with the fields lx, ly, lz, nw, xbits, ybits, rowtab, Nf.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.cuh"

namespace lbg {

// AA layout over the fluid nodes: compact index of the fluid node x of the lattice row whose
// table entries start at rb, from the row's fluid bitmask word and the compact index of its
// first fluid node.
__device__ __forceinline__ unsigned compact_in_row(const uint2 *__restrict__ rowtab, unsigned rb, int x)
{
    const uint2 e = __ldg(rowtab + rb + (x >> 5));
    return e.y + (unsigned)__popc(e.x & ((1u << (x & 31)) - 1u));
}

// Compact node position: x | y << xbits | z << (xbits + ybits) (no division to decode).
template <typename A>
__device__ __forceinline__ unsigned lattice_of(const A &a, unsigned c)
{
    const unsigned x = c & ((1u << a.xbits) - 1u);
    const unsigned y = (c >> a.xbits) & ((1u << a.ybits) - 1u);
    const unsigned z = c >> (a.xbits + a.ybits);
    return x + (unsigned)a.lx * (y + (unsigned)a.ly * z);
}

// Element index of the slot read for each direction by the gather of an odd AA launch at the
// compact node i (packed position c, flag word m): slot l of the node itself across a bounce-back
// link, else slot inv(l) of the fluid node x - c_l (the reference's halfway bounce-back and
// streaming, equilibration.f90:204-243, in pull form).  f(l, o) is called for every l.
// Within a lattice row the fluid nodes are consecutive compact indices, so one table lookup per
// neighbouring row gives cnt = the compact index the node x would have in that row (fluid nodes
// before x); its neighbours x -+ 1 in the row are then cnt - 1 and cnt + fluid(x) (x - 1 and
// x + 1 fluid), and the node's own row needs no lookup (cnt = i).  The eight lookups are made
// up front, independent of the bounce-back bits, so that they are in flight together and each
// serves every direction into its row; only a wrap across the periodic x boundary takes a second
// lookup.  Off: the type of the offsets (unsigned while 19 Nf < 2^32, else 64-bit).
template <typename Off = unsigned, typename A, typename Fn>
__device__ __forceinline__ void aa_gather_offsets(const A &a, unsigned i, unsigned c,
                                                  uint32_t m, Fn &&f)
{
    const int lx = a.lx, ly = a.ly, lz = a.lz, nw = a.nw;
    const int x = (int)(c & ((1u << a.xbits) - 1u));
    const int y = (int)((c >> a.xbits) & ((1u << a.ybits) - 1u));
    const int z = (int)(c >> (a.xbits + a.ybits));
    const unsigned row = (unsigned)(y + ly * z);
    // [c+1] = row coordinate of (y - c), (z - c)
    const int R[3] = {wrap_plus(y, ly), y, wrap_minus(y, ly)};
    const int Z[3] = {wrap_plus(z, lz) * ly, z * ly, wrap_minus(z, lz) * ly};
    const unsigned Nf = a.Nf;
    const int w = x >> 5, b = x & 31;
    const uint32_t below = (1u << b) - 1u;
    const uint2 *__restrict__ tab = a.rowtab;
    // neighbouring rows, slot k = 3 (c.y + 1) + (c.z + 1) (k = 4: the node's own row)
    uint2 e[9];
    static_for<0, 9>([&](auto K) {
        constexpr int k = decltype(K)::value;
        if constexpr (k != 4) e[k] = __ldg(tab + (unsigned)(R[k / 3] + Z[k % 3]) * (unsigned)nw + w);
    });
    static_for<0, Q>([&](auto L) {
        constexpr int l = decltype(L)::value;
        constexpr Vel v = vel(l);
        if constexpr (l == 0) {
            f(0, (Off)i);
        } else {
            constexpr int k = 3 * (v.y + 1) + (v.z + 1);
            unsigned s;
            if constexpr (k == 4) {
                // own row: the fluid neighbour x - c.x is the previous / next compact node
                const unsigned rb = row * (unsigned)nw;
                if constexpr (v.x > 0) s = x > 0 ? i - 1u : compact_in_row(tab, rb, lx - 1);
                else s = x < lx - 1 ? i + 1u : compact_in_row(tab, rb, 0);
            } else {
                const unsigned cnt = e[k].y + (unsigned)__popc(e[k].x & below);
                if constexpr (v.x == 0) {
                    s = cnt;
                } else {
                    const unsigned rb = (unsigned)(R[v.y + 1] + Z[v.z + 1]) * (unsigned)nw;
                    if constexpr (v.x > 0) s = x > 0 ? cnt - 1u : compact_in_row(tab, rb, lx - 1);
                    else s = x < lx - 1 ? cnt + ((e[k].x >> b) & 1u) : compact_in_row(tab, rb, 0);
                }
            }
            f(l, ((m >> l) & 1u) ? (Off)l * Nf + i : (Off)inv(l) * Nf + s);
        }
    });
}

// Host: tables of the compact layout of a box from its nature array (0 = fluid).  Returns false
// when the packed positions do not fit 32 bits.
inline bool build_compact_tables(int lx, int ly, int lz, const int8_t *nature, std::vector<uint2> &rowtab,
                                 std::vector<uint32_t> &pos, int &nw, int &xbits, int &ybits)
{
    auto bits = [](int n) {
        int b = 1;
        while ((1 << b) < n) ++b;
        return b;
    };
    xbits = bits(lx);
    ybits = bits(ly);
    const int zbits = bits(lz);
    nw = (lx + 31) / 32;
    const long long rows = (long long)ly * lz;
    if (xbits + ybits + zbits > 32 || rows * nw >= (1LL << 32)) return false;
    rowtab.assign((size_t)rows * nw, make_uint2(0u, 0u));
    pos.clear();
    uint32_t c = 0;
    for (int z = 0; z < lz; ++z)
        for (int y = 0; y < ly; ++y) {
            const size_t r = (size_t)y + (size_t)ly * z;
            for (int w = 0; w < nw; ++w) {
                uint32_t bm = 0;
                const uint32_t base = c;
                for (int b = 0; b < 32; ++b) {
                    const int x = w * 32 + b;
                    if (x < lx && nature[r * lx + x] == 0) {
                        bm |= 1u << b;
                        pos.push_back((uint32_t)x | ((uint32_t)y << xbits) | ((uint32_t)z << (xbits + ybits)));
                        ++c;
                    }
                }
                rowtab[r * nw + w] = make_uint2(bm, base);
            }
        }
    return true;
}

}  // namespace lbg
