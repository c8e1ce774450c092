// batch_api.cu -- C ABI of batches of boxes and of the request server built on them.
//
// A batch owns any number of boxes (slots) of any size, each with one device allocation taken
// from the stream-ordered pool.  Boxes can be added and removed and change phase between
// calls; the descriptor table and the work lists are rebuilt on the next call and one call's
// launches are replayed from a CUDA graph.  lbgpu_serve runs a request loop on a batch:
// requests are admitted when they have arrived and their buffers fit the memory budget, stay
// resident and are stepped together with whatever else is resident, and leave as soon as
// their own convergence test (or step cap) and tracer steps are done -- continuous batching.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "batch.h"
#include "compact.cuh"
#include "ctx.h"
#include "flow.h"
#include "lbgpu.h"
#include "trace.h"

using namespace lbg;

namespace {

constexpr double EPS = 2.220446049250313e-16;  // epsilon(1._dp)
constexpr size_t ALIGN = 256;

struct Slot {
    bool active = false;
    BatchInst d{};            // device descriptor (pointers into this slot's allocation)
    void *mem = nullptr;      // the slot's one device allocation
    long long fluid = 0;
    size_t bytes = 0;
    bool smem = false;        // stepped with the whole box in shared memory (lattice layout)
    bool tracer = false;
    int ntile = 0;            // tiles with VACF accumulators (256-node tiles or slab tiles)
    int mp_steps = 0;
    // slab tiles of the tracer phase that hold a fluid node (a tile of solid nodes only has
    // nothing to step: it writes no P and adds nothing to the VACF, whose accumulators start at 0)
    std::vector<int> slab_live;
};

struct GraphEntry {
    int nsteps = 0;
    bool check = false;
    bool smem = false;   // holds the shared-memory boxes' launch
    cudaGraphExec_t exec = nullptr;
};

size_t up(size_t x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

bool tracer_ads(const lbgpu_tracer &t)
{
    const double K = std::fabs(t.kd) <= EPS ? 0.0 : t.ka / t.kd;
    return std::fabs(K) > EPS;
}

// Byte layout of a slot's allocation: populations (g, over `units` nodes: lattice nodes, or
// fluid nodes in the compact layout), lattice flags, previous velocity per unit, nature, the
// compact tables (positions, flags, row table of `tab` entries) and the tracer buffers
// (lattice-ordered V, P, A, the fixed (u*, D) and per-tile VACF accumulators).
struct Layout {
    size_t g, mask, uprev, nature, cpos, cmask, rowtab, V, P0, P1, A0, A1, aux, tacc, total;
};

Layout layout(long long N, long long units, long long tab, long long ntacc, bool compact, bool tracer,
              bool ads)
{
    Layout L{};
    size_t o = 0;
    L.g = o;      o += up(sizeof(float) * Q * (size_t)units);
    L.mask = o;   o += up(sizeof(uint32_t) * (size_t)N);
    L.uprev = o;  o += up(sizeof(float4) * (size_t)units);
    L.nature = o; o += up((size_t)N);
    if (compact) {
        L.cpos = o;   o += up(sizeof(uint32_t) * (size_t)units);
        L.cmask = o;  o += up(sizeof(uint32_t) * (size_t)units);
        L.rowtab = o; o += up(sizeof(uint2) * (size_t)tab);
    }
    if (tracer) {
        const size_t f4 = up(sizeof(float4) * (size_t)N);
        L.V = o;  o += f4;
        L.P0 = o; o += f4;
        L.P1 = o; o += f4;
        if (ads) {
            L.A0 = o; o += f4;
            L.A1 = o; o += f4;
        }
        L.aux = o; o += f4;
        L.tacc = o; o += up(sizeof(double) * ((size_t)ntacc * BATCH_TACC + 1));
    }
    L.total = o;
    return L;
}

// Upper bound of a box's footprint over both layouts (the fluid count is not known before the
// geometry is read): the lattice layout plus the compact tables for every node.
size_t footprint_bound(long long N, int lx, int ly, int lz, bool tracer, bool ads)
{
    const long long tab = (long long)ly * lz * ((lx + 31) / 32);
    const long long ntacc = std::max<long long>((N + BATCH_BLOCK - 1) / BATCH_BLOCK, batch_slab_tiles(lx, ly, lz));
    return layout(N, N, tab, ntacc, true, tracer, ads).total;
}

}  // namespace

struct lbgpu_batch {
    int device = 0;
    // side: the shared-memory boxes in the flow phase, side2: those in the tracer phase, side3:
    // the tiled boxes in the tracer phase while tiled boxes are also in the flow phase
    cudaStream_t stream = nullptr, side = nullptr, side2 = nullptr, side3 = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr, join = nullptr, join2 = nullptr;
    cudaEvent_t fork_mp = nullptr, join_mp = nullptr;
    size_t budget = 0, used = 0;
    int smem_max = BATCH_SMEM_BYTES_MAX;
    std::vector<Slot> slots;
    unsigned long long *d_counts = nullptr;
    // device tables, rebuilt when the set of boxes or a phase changes
    bool dirty = true;
    BatchInst *d_insts = nullptr;
    int cap_insts = 0;
    BatchTile *d_tiles = nullptr;   // flow tiles, then tracer tiles, then tracer slab tiles
    int cap_tiles = 0, nflow = 0, nmp = 0, nslab = 0;
    int *d_smem = nullptr;
    // shared-memory boxes: the flow-phase ones first (nsmem_flow), each phase with its bytes
    int cap_smem = 0, nsmem = 0, nsmem_flow = 0, smem_bytes_flow = 0, smem_bytes_mp = 0;
    int smem_threads = BATCH_SMEM_THREADS;
    unsigned *d_du = nullptr;
    int cap_du = 0;
    int aa_minb[2] = {4, 5};      // resident blocks per SM of the even / odd AA launches
    // work-list form of the even / odd AA launch (a persistent grid claiming tiles from a ticket)
    // and the tiles a block claims at a time; 0: one block per tile
    int aa_list[2] = {0, 0}, aa_tpc[2] = {1, 1};
    float aa_ms[2] = {0.0f, 0.0f};    // measured time of one launch of the chosen variants
    long long tuned_fluid = 0;        // fluid nodes of the flow-phase tiled boxes they were timed on
    int steps_per_graph = 0;          // 0: one graph per call (before the tuner ran)
    int sms = 0;
    BatchTicket *d_ticket = nullptr;
    bool aa_tuned = false;
    bool smem_tuned = false;
    std::vector<int> desc_slot;   // descriptor index -> slot
    std::vector<GraphEntry> graphs;
};

namespace {

int bfail(int code, const std::string &msg) { return ctx_fail(nullptr, code, msg); }

#define LBB_CK(call)                                                                   \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) return bfail(LBGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
int grow(T **p, int &cap, int need, cudaStream_t s)
{
    if (need <= cap) return LBGPU_OK;
    int nc = std::max(need, cap * 2 + 16);
    if (*p) LBB_CK(cudaFreeAsync(*p, s));
    LBB_CK(cudaMallocAsync((void **)p, sizeof(T) * nc, s));
    cap = nc;
    return LBGPU_OK;
}

void drop_graphs(lbgpu_batch *b)
{
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.exec);
    b->graphs.clear();
}

void fill_consts(BatchInst &d, const lbgpu_cell &c)
{
    const LbConst64 K = make_const64(c.relaxation_time);
    const double c2 = K.c2, c3 = K.c3, cs2 = 1.0 / 3.0;
    d.c1 = (float)K.c1;
    for (int w = 0; w < 3; ++w) {
        d.c2w[w] = (float)(c2 * K.a0[w]);
        d.c2a1[w] = (float)(c2 * K.a1[w]);
        d.c2a2[w] = (float)(c2 * K.a2[w]);
        d.c2a2cs2[w] = (float)(c2 * K.a2[w] * cs2);
        d.c3a1[w] = (float)(c3 * K.a1[w]);
    }
    for (int p = 0; p < 9; ++p) {
        const int l = pair_l(p);
        const Vel v = vel(l);
        const double cF = v.x * c.f_ext[0] + v.y * c.f_ext[1] + v.z * c.f_ext[2];
        d.kF[p] = (float)(c3 * K.a1[wclass(l)] * cF);
        d.kT[p] = (float)(c3 * K.two_a2[wclass(l)] * cF);
    }
    for (int q = 0; q < 3; ++q) d.F[q] = (float)c.f_ext[q];
    d.rho0 = (float)c.rho0;
    d.force = (c.f_ext[0] != 0.0 || c.f_ext[1] != 0.0 || c.f_ext[2] != 0.0) ? 1 : 0;
    // tracer constants as in mp_api.cu (module_moment_propagation.f90:331-337)
    const lbgpu_tracer &t = c.tracer;
    const volatile double kBT = 1.0 / 3.0;
    const double lambda = 4.0 * t.Db / kBT;
    for (int w = 0; w < 3; ++w) {
        d.a1[w] = (float)K.a1[w];
        const volatile double lw = lambda * K.a0[w];
        d.lwh[w] = (float)(lw * 0.5);
    }
    d.ka = (float)t.ka;
    d.kd = (float)t.kd;
    d.one_minus_kd = (float)(1.0 - t.kd);
    for (int q = 0; q < 3; ++q) d.tfext[q] = t.f_ext[q];
}

int rebuild(lbgpu_batch *b)
{
    if (!b->dirty) return LBGPU_OK;
    cudaStream_t s = b->stream;
    drop_graphs(b);
    std::vector<BatchInst> descs;
    std::vector<BatchTile> flow, mp, slab;
    std::vector<int> smem, smem_mp;
    b->desc_slot.clear();
    int bytes_flow = 0, bytes_mp = 0;
    for (size_t k = 0; k < b->slots.size(); ++k) {
        const Slot &sl = b->slots[k];
        if (!sl.active) continue;
        const int id = (int)descs.size();
        descs.push_back(sl.d);
        b->desc_slot.push_back((int)k);
        if (sl.smem) {
            if (sl.d.phase == BATCH_FLOW) {
                smem.push_back(id);
                bytes_flow = std::max(bytes_flow, batch_smem_flow(sl.d.N));
            } else {
                smem_mp.push_back(id);
                bytes_mp = std::max(bytes_mp, batch_smem_mp(sl.d.N, sl.d.ads));
            }
        } else if (sl.d.phase == BATCH_MP && sl.d.zc > 0) {
            for (int k : sl.slab_live) slab.push_back({id, k});
        } else {
            auto &list = sl.d.phase == BATCH_FLOW ? flow : mp;
            const int units = (int)batch_units(sl.d);
            for (int st = 0; st < units; st += BATCH_BLOCK) list.push_back({id, st});
        }
    }
    const int nsmem_flow = (int)smem.size();
    smem.insert(smem.end(), smem_mp.begin(), smem_mp.end());
    std::vector<BatchTile> tiles(flow);
    tiles.insert(tiles.end(), mp.begin(), mp.end());
    tiles.insert(tiles.end(), slab.begin(), slab.end());
    int rc;
    if ((rc = grow(&b->d_insts, b->cap_insts, (int)descs.size(), s))) return rc;
    if ((rc = grow(&b->d_tiles, b->cap_tiles, (int)tiles.size(), s))) return rc;
    if ((rc = grow(&b->d_smem, b->cap_smem, (int)smem.size(), s))) return rc;
    if ((rc = grow(&b->d_du, b->cap_du, std::max<int>((int)descs.size(), 1), s))) return rc;
    if (!descs.empty())
        LBB_CK(cudaMemcpyAsync(b->d_insts, descs.data(), sizeof(BatchInst) * descs.size(), cudaMemcpyHostToDevice, s));
    if (!tiles.empty())
        LBB_CK(cudaMemcpyAsync(b->d_tiles, tiles.data(), sizeof(BatchTile) * tiles.size(), cudaMemcpyHostToDevice, s));
    if (!smem.empty())
        LBB_CK(cudaMemcpyAsync(b->d_smem, smem.data(), sizeof(int) * smem.size(), cudaMemcpyHostToDevice, s));
    LBB_CK(cudaStreamSynchronize(s));  // host vectors above go out of scope
    b->nflow = (int)flow.size();
    b->nmp = (int)mp.size();
    b->nslab = (int)slab.size();
    b->nsmem = (int)smem.size();
    b->nsmem_flow = nsmem_flow;
    b->smem_bytes_flow = bytes_flow;
    b->smem_bytes_mp = bytes_mp;
    b->dirty = false;
    return LBGPU_OK;
}

// One AA launch of the flow-phase tiles in the variant the tuner chose (descriptors insts: the
// batch's, or the tuner's scratch copies).
int launch_aa(lbgpu_batch *b, const BatchInst *insts, int odd, cudaStream_t s)
{
    if (b->aa_list[odd])
        LBB_CK(launch_batch_aa_list(insts, b->d_tiles, b->nflow, odd, b->aa_minb[odd], b->sms * b->aa_minb[odd],
                                    b->aa_tpc[odd], b->d_ticket, s));
    else
        LBB_CK(launch_batch_aa(insts, b->d_tiles, b->nflow, odd, b->aa_minb[odd], s));
    return LBGPU_OK;
}

// The shared-memory boxes' launches for nsteps steps, forked from the main stream: the flow-phase
// boxes on the side stream and the tracer-phase ones on the second side stream, concurrently (one
// block per box, on disjoint boxes; in sequence a call of a batch in both phases cost the sum of
// the two).  The main stream waits for both (join_smem).
int enqueue_smem(lbgpu_batch *b, int nsteps, bool check)
{
    const int nflow = b->nsmem_flow, nmp = b->nsmem - b->nsmem_flow;
    LBB_CK(cudaEventRecord(b->fork, b->stream));
    LBB_CK(cudaStreamWaitEvent(b->side, b->fork, 0));
    LBB_CK(cudaStreamWaitEvent(b->side2, b->fork, 0));
    LBB_CK(launch_batch_smem(b->d_insts, b->d_smem, nflow, 0, nsteps, check, b->d_du, b->smem_bytes_flow,
                             b->smem_bytes_mp, b->smem_threads, b->side));
    LBB_CK(launch_batch_smem(b->d_insts, b->d_smem + nflow, 0, nmp, nsteps, check, b->d_du, b->smem_bytes_flow,
                             b->smem_bytes_mp, b->smem_threads, b->side2));
    LBB_CK(cudaEventRecord(b->join, b->side));
    LBB_CK(cudaEventRecord(b->join2, b->side2));
    return LBGPU_OK;
}

int join_smem(lbgpu_batch *b)
{
    LBB_CK(cudaStreamWaitEvent(b->stream, b->join, 0));
    LBB_CK(cudaStreamWaitEvent(b->stream, b->join2, 0));
    return LBGPU_OK;
}

int clear_du(lbgpu_batch *b)
{
    LBB_CK(cudaMemsetAsync(b->d_du, 0, sizeof(unsigned) * std::max<size_t>(b->desc_slot.size(), 1), b->stream));
    return LBGPU_OK;
}

// The launches of one call (or, with smem = false, of a part of a call whose shared-memory boxes
// run in a launch of their own): the shared-memory boxes on the side streams, concurrently with the
// per-step launches of the tiled boxes: those of the flow-phase boxes on the main stream and, when
// both phases hold tiled boxes, those of the tracer-phase boxes as a second chain on the third
// side stream (the two chains step disjoint boxes and meet at the end of the call).
int enqueue_steps(lbgpu_batch *b, int nsteps, bool check, bool smem)
{
    cudaStream_t s = b->stream;
    if (check && smem)
        if (int rc = clear_du(b)) return rc;
    if (b->nsmem && smem)
        if (int rc = enqueue_smem(b, nsteps, check)) return rc;
    const bool flow_tiles = b->nflow > 0, mp_tiles = b->nmp + b->nslab > 0;
    cudaStream_t ms = s;
    if (flow_tiles && mp_tiles) {
        LBB_CK(cudaEventRecord(b->fork_mp, s));
        LBB_CK(cudaStreamWaitEvent(b->side3, b->fork_mp, 0));
        ms = b->side3;
    }
    for (int t = 0; t < nsteps; ++t) {
        if (flow_tiles)
            if (int rc = launch_aa(b, b->d_insts, t & 1, s)) return rc;
        if (mp_tiles) {
            LBB_CK(launch_batch_mp(b->d_insts, b->d_tiles + b->nflow, b->nmp, t & 1, ms));
            LBB_CK(launch_batch_mp_slab(b->d_insts, b->d_tiles + b->nflow + b->nmp, b->nslab, t & 1, ms));
        }
    }
    if (ms != s) {
        LBB_CK(cudaEventRecord(b->join_mp, ms));
        LBB_CK(cudaStreamWaitEvent(s, b->join_mp, 0));
    }
    if (check) LBB_CK(launch_batch_check(b->d_insts, b->d_tiles, b->nflow, b->d_du, s));
    if (b->nsmem && smem)
        if (int rc = join_smem(b)) return rc;
    return LBGPU_OK;
}

// The graph of one call (nsteps, check), captured on first use and kept until the batch's
// tables change.
int graph_of(lbgpu_batch *b, int nsteps, bool check, bool smem, cudaGraphExec_t *out)
{
    for (auto &g : b->graphs)
        if (g.nsteps == nsteps && g.check == check && g.smem == smem) {
            *out = g.exec;
            return LBGPU_OK;
        }
    cudaStream_t s = b->stream;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    LBB_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_steps(b, nsteps, check, smem);
    const cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (rc) {
        if (e == cudaSuccess) cudaGraphDestroy(graph);
        return rc;
    }
    LBB_CK(e);
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    LBB_CK(ei);
    if (b->graphs.size() >= 4) {
        cudaGraphExecDestroy(b->graphs.front().exec);
        b->graphs.erase(b->graphs.begin());
    }
    b->graphs.push_back({nsteps, check, smem, exec});
    *out = exec;
    return LBGPU_OK;
}

// Tuner of the tiled AA launches: the first time a batch holds at least 1024 flow tiles, every
// variant of the even and of the odd launch is timed on scratch copies of the tiled boxes'
// populations (a second descriptor table points at them; the boxes' state is not advanced) and
// the fastest is kept for the batch's lifetime: one block per tile at 3..6 resident blocks per
// SM, or the persistent work list (4..6 blocks per SM claiming 1, 2 or 4 tiles at a time from an
// atomic ticket).  It then picks the steps per graph (see below).
// LBGPU_BATCH_AA_MINB=<even>,<odd> fixes one-block-per-tile variants instead, and
// LBGPU_BATCH_AA_LIST=<blocks per SM>,<tiles per claim>[,<steps per graph>] the work-list form
// of both launches (for any number of tiles).
int tune_aa(lbgpu_batch *b)
{
    if (b->aa_tuned) return LBGPU_OK;
    if (const char *e = std::getenv("LBGPU_BATCH_AA_LIST")) {
        int minb = 0, tpc = 0, spg = 0;
        const int n = std::sscanf(e, "%d,%d,%d", &minb, &tpc, &spg);
        if (n >= 2 && minb >= 3 && minb <= 6 && tpc >= 1) {
            b->aa_tuned = true;
            for (int k = 0; k < 2; ++k) {
                b->aa_list[k] = 1;
                b->aa_minb[k] = minb;
                b->aa_tpc[k] = tpc;
            }
            if (n == 3 && spg > 0 && spg % 2 == 0) b->steps_per_graph = spg;
            drop_graphs(b);
            return LBGPU_OK;
        }
    }
    if (b->nflow < 1024) return LBGPU_OK;
    b->aa_tuned = true;
    if (const char *e = std::getenv("LBGPU_BATCH_AA_MINB")) {
        int ev = 0, od = 0;
        if (std::sscanf(e, "%d,%d", &ev, &od) == 2) {
            b->aa_minb[0] = ev;
            b->aa_minb[1] = od;
            return LBGPU_OK;
        }
    }
    cudaStream_t s = b->stream;
    std::vector<BatchInst> descs(b->desc_slot.size());
    size_t total = 0;
    for (size_t i = 0; i < descs.size(); ++i) {
        descs[i] = b->slots[b->desc_slot[i]].d;
        if (!descs[i].compact || descs[i].phase != BATCH_FLOW) continue;
        total += (size_t)Q * descs[i].Nf;
    }
    float *scratch = nullptr;
    BatchInst *d_tmp = nullptr;
    if (cudaMallocAsync(&scratch, sizeof(float) * total, s) != cudaSuccess ||
        cudaMallocAsync(&d_tmp, sizeof(BatchInst) * descs.size(), s) != cudaSuccess) {
        cudaGetLastError();   // no room: keep the default variants
        if (scratch) cudaFreeAsync(scratch, s);
        return LBGPU_OK;
    }
    size_t off = 0;
    for (auto &d : descs) {
        if (!d.compact || d.phase != BATCH_FLOW) continue;
        LBB_CK(cudaMemcpyAsync(scratch + off, d.g, sizeof(float) * Q * d.Nf, cudaMemcpyDeviceToDevice, s));
        d.g = scratch + off;
        off += (size_t)Q * d.Nf;
    }
    LBB_CK(cudaMemcpyAsync(d_tmp, descs.data(), sizeof(BatchInst) * descs.size(), cudaMemcpyHostToDevice, s));
    // candidates of each launch: one block per tile at 3..6 resident blocks per SM, and the
    // persistent work list at 4..6 blocks per SM claiming 1, 2 or 4 tiles at a time
    struct Cand {
        int list, minb, tpc;
    };
    std::vector<Cand> cands;
    for (int minb = 3; minb <= 6; ++minb) cands.push_back({0, minb, 1});
    for (int minb = 4; minb <= 6; ++minb)
        for (int tpc : {1, 2, 4}) cands.push_back({1, minb, tpc});
    long long fluid = 0;
    for (const auto &d : descs)
        if (d.compact && d.phase == BATCH_FLOW) fluid += d.Nf;
    for (int odd = 0; odd < 2; ++odd) {
        float best = 1e30f;
        Cand keep = cands[0];
        for (const Cand &c : cands) {
            b->aa_list[odd] = c.list;
            b->aa_minb[odd] = c.minb;
            b->aa_tpc[odd] = c.tpc;
            for (int k = 0; k < 2; ++k)
                if (int rc = launch_aa(b, d_tmp, odd, s)) return rc;
            LBB_CK(cudaEventRecord(b->ev0, s));
            for (int k = 0; k < 6; ++k)
                if (int rc = launch_aa(b, d_tmp, odd, s)) return rc;
            LBB_CK(cudaEventRecord(b->ev1, s));
            LBB_CK(cudaEventSynchronize(b->ev1));
            float ms = 0.0f;
            LBB_CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
            if (ms < best) {
                best = ms;
                keep = c;
            }
        }
        b->aa_list[odd] = keep.list;
        b->aa_minb[odd] = keep.minb;
        b->aa_tpc[odd] = keep.tpc;
        b->aa_ms[odd] = best / 6.0f;
    }
    b->tuned_fluid = fluid;
    // steps per graph: a call's steps run as graphs of S steps (the last one holds the rest); S
    // is the smallest of 8, 32, 128 whose 128 steps (AA launches on the scratch copies) take no
    // more than 1 % longer than the fastest S (graph launches cost a few microseconds, while a
    // smaller S lets the host act sooner on a long call and keeps the graphs small).  The tuning
    // runs inside the first call, so it is kept short: about 550 launches.
    {
        constexpr int NS = 3, TS = 128;
        float tS[NS];
        const int Ss[NS] = {8, 32, 128};
        for (int q = 0; q < NS; ++q) {
            cudaGraph_t g;
            cudaGraphExec_t ex;
            LBB_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            int rc = LBGPU_OK;
            for (int t = 0; t < Ss[q] && !rc; ++t) rc = launch_aa(b, d_tmp, t & 1, s);
            const cudaError_t ce = cudaStreamEndCapture(s, &g);
            if (rc) {
                if (ce == cudaSuccess) cudaGraphDestroy(g);
                return rc;
            }
            LBB_CK(ce);
            const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            LBB_CK(ie);
            LBB_CK(cudaGraphLaunch(ex, s));   // warm-up
            LBB_CK(cudaEventRecord(b->ev0, s));
            for (int k = 0; k < TS / Ss[q]; ++k) LBB_CK(cudaGraphLaunch(ex, s));
            LBB_CK(cudaEventRecord(b->ev1, s));
            LBB_CK(cudaEventSynchronize(b->ev1));
            LBB_CK(cudaEventElapsedTime(&tS[q], b->ev0, b->ev1));
            cudaGraphExecDestroy(ex);
        }
        const float fastest = *std::min_element(tS, tS + NS);
        for (int q = 0; q < NS; ++q)
            if (tS[q] <= 1.01f * fastest) {
                b->steps_per_graph = Ss[q];
                break;
            }
    }
    LBB_CK(cudaFreeAsync(scratch, s));
    LBB_CK(cudaFreeAsync(d_tmp, s));
    LBB_CK(cudaStreamSynchronize(s));   // descs go out of scope
    drop_graphs(b);                     // graphs captured with the previous variants
    return LBGPU_OK;
}

// Block-size tuner of the shared-memory kernel: the first time a batch holds at least 64
// shared-memory boxes, all in the flow phase, 20 steps are timed twice with 256 and with 512
// threads per box on scratch copies of their populations (the boxes' state does not advance) and
// the fastest is kept.  (1024 threads, at most 64 registers each, spill and lose in the tracer
// phase, which cannot be timed before the flow has run; LBGPU_BATCH_SMEM_THREADS=1024 still
// selects them.)  LBGPU_BATCH_SMEM_THREADS fixes the size instead.
int tune_smem(lbgpu_batch *b)
{
    if (b->smem_tuned || b->nsmem < 64) return LBGPU_OK;
    b->smem_tuned = true;
    if (const char *e = std::getenv("LBGPU_BATCH_SMEM_THREADS")) {
        const int t = std::atoi(e);
        if (t == 256 || t == 512 || t == 1024) b->smem_threads = t;
        return LBGPU_OK;
    }
    std::vector<BatchInst> descs(b->desc_slot.size());
    size_t total = 0;
    for (size_t i = 0; i < descs.size(); ++i) {
        const Slot &sl = b->slots[b->desc_slot[i]];
        descs[i] = sl.d;
        if (!sl.smem) continue;
        if (sl.d.phase != BATCH_FLOW) return LBGPU_OK;
        total += (size_t)Q * sl.d.N;
    }
    cudaStream_t s = b->stream;
    float *scratch = nullptr;
    BatchInst *d_tmp = nullptr;
    if (cudaMallocAsync(&scratch, sizeof(float) * total, s) != cudaSuccess ||
        cudaMallocAsync(&d_tmp, sizeof(BatchInst) * descs.size(), s) != cudaSuccess) {
        cudaGetLastError();   // no room: keep the default
        if (scratch) cudaFreeAsync(scratch, s);
        return LBGPU_OK;
    }
    size_t off = 0;
    for (size_t i = 0; i < descs.size(); ++i) {
        if (!b->slots[b->desc_slot[i]].smem) continue;
        BatchInst &d = descs[i];
        LBB_CK(cudaMemcpyAsync(scratch + off, d.g, sizeof(float) * Q * d.N, cudaMemcpyDeviceToDevice, s));
        d.g = scratch + off;
        off += (size_t)Q * d.N;
    }
    LBB_CK(cudaMemcpyAsync(d_tmp, descs.data(), sizeof(BatchInst) * descs.size(), cudaMemcpyHostToDevice, s));
    const int cand[2] = {256, 512};
    float best[2] = {1e30f, 1e30f};
    for (int rep = 0; rep < 2; ++rep)
        for (int k = 0; k < 2; ++k) {
            LBB_CK(launch_batch_smem(d_tmp, b->d_smem, b->nsmem, 0, 2, false, nullptr, b->smem_bytes_flow, 0,
                                     cand[k], s));
            LBB_CK(cudaEventRecord(b->ev0, s));
            LBB_CK(launch_batch_smem(d_tmp, b->d_smem, b->nsmem, 0, 20, false, nullptr, b->smem_bytes_flow, 0,
                                     cand[k], s));
            LBB_CK(cudaEventRecord(b->ev1, s));
            LBB_CK(cudaEventSynchronize(b->ev1));
            float ms = 0.0f;
            LBB_CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
            best[k] = std::min(best[k], ms);
        }
    b->smem_threads = best[0] < best[1] ? cand[0] : cand[1];
    LBB_CK(cudaFreeAsync(scratch, s));
    LBB_CK(cudaFreeAsync(d_tmp, s));
    LBB_CK(cudaStreamSynchronize(s));   // descs go out of scope
    drop_graphs(b);
    return LBGPU_OK;
}

// A call's steps run as graphs of steps_per_graph steps (the tuner's choice), the last one with
// the rest and the convergence check.  The shared-memory boxes step the whole call in one launch
// whatever the split (each of their launches loads and stores the boxes once): inside the graph
// when the call is one graph, else launched on its own before the graphs, which then hold only
// the tiled boxes' launches.  launch = false only captures the graphs.
int call_graphs(lbgpu_batch *b, int nsteps, bool check, bool launch)
{
    const int S = b->steps_per_graph > 0 ? b->steps_per_graph : nsteps;
    const bool split = S < nsteps && b->nsmem > 0;
    if (split && launch) {
        if (check)
            if (int rc = clear_du(b)) return rc;
        if (int rc = enqueue_smem(b, nsteps, check)) return rc;
    }
    int left = nsteps;
    while (left > 0) {
        const int n = left > S ? S : left;
        left -= n;
        cudaGraphExec_t exec = nullptr;
        if (int rc = graph_of(b, n, check && left == 0, !split, &exec)) return rc;
        if (launch) LBB_CK(cudaGraphLaunch(exec, b->stream));
    }
    if (split && launch)
        if (int rc = join_smem(b)) return rc;
    return LBGPU_OK;
}

int run_steps(lbgpu_batch *b, int nsteps, bool check)
{
    if (int rc = tune_aa(b)) return rc;
    if (int rc = tune_smem(b)) return rc;
    if (int rc = call_graphs(b, nsteps, check, true)) return rc;
    for (auto &sl : b->slots)
        if (sl.active && sl.d.phase == BATCH_MP) sl.mp_steps += nsteps;
    return LBGPU_OK;
}

int desc_of(lbgpu_batch *b, int id)
{
    for (size_t i = 0; i < b->desc_slot.size(); ++i)
        if (b->desc_slot[i] == id) return (int)i;
    return -1;
}

bool valid_slot(lbgpu_batch *b, int id)
{
    return b && id >= 0 && id < (int)b->slots.size() && b->slots[id].active;
}

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

size_t lbgpu_batch_footprint(const lbgpu_cell *c)
{
    if (!c || c->lx <= 0 || c->ly <= 0 || c->lz <= 0) return 0;
    const long long N = (long long)c->lx * c->ly * c->lz;
    const bool tracer = c->tracer.Db != 0.0;
    return footprint_bound(N, c->lx, c->ly, c->lz, tracer, tracer && tracer_ads(c->tracer));
}

int lbgpu_batch_create(int device, size_t memory_budget, lbgpu_batch **out)
{
    if (!out) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_create: null argument");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return bfail(LBGPU_ERR_CUDA, "no CUDA device");
    if (device < 0 || device >= ndev) return bfail(LBGPU_ERR_INVALID, "bad device ordinal");
    LBB_CK(cudaSetDevice(device));
    lbgpu_batch *b = new lbgpu_batch();
    b->device = device;
    size_t fr = 0, tot = 0;
    e = cudaMemGetInfo(&fr, &tot);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side2, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side3, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join2, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork_mp, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join_mp, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_counts, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void **)&b->d_ticket, sizeof(BatchTicket));
    if (e == cudaSuccess) e = cudaMemset(b->d_ticket, 0, sizeof(BatchTicket));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    int optin = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e == cudaSuccess) {
        // the shared-memory kernel also holds a small static reduction buffer
        b->smem_max = std::min(b->smem_max, optin) - 1024;
        e = batch_configure(b->smem_max);
    }
    if (e != cudaSuccess) {
        lbgpu_batch_destroy(b);
        return bfail(LBGPU_ERR_CUDA, std::string("lbgpu_batch_create: ") + cudaGetErrorString(e));
    }
    b->budget = memory_budget ? memory_budget : (size_t)(0.9 * (double)fr);
    // LBGPU_BATCH_SMEM=0 steps every box with the tiled kernels (same per-node arithmetic)
    const char *mode = std::getenv("LBGPU_BATCH_SMEM");
    if (mode && std::string(mode) == "0") b->smem_max = 0;
    *out = b;
    return LBGPU_OK;
}

void lbgpu_batch_destroy(lbgpu_batch *b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->side) cudaStreamSynchronize(b->side);
    if (b->side2) cudaStreamSynchronize(b->side2);
    if (b->side3) cudaStreamSynchronize(b->side3);
    drop_graphs(b);
    for (auto &sl : b->slots)
        if (sl.active) cudaFree(sl.mem);
    cudaFree(b->d_insts);
    cudaFree(b->d_tiles);
    cudaFree(b->d_smem);
    cudaFree(b->d_du);
    cudaFree(b->d_counts);
    cudaFree(b->d_ticket);
    for (cudaEvent_t ev : {b->ev0, b->ev1, b->fork, b->join, b->join2, b->fork_mp, b->join_mp})
        if (ev) cudaEventDestroy(ev);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->side2) cudaStreamDestroy(b->side2);
    if (b->side3) cudaStreamDestroy(b->side3);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int lbgpu_batch_add_label(lbgpu_batch *b, const lbgpu_cell *c, int label, const double *params, int *id)
{
    if (!b || !c || !id) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_add_label: null argument");
    if (c->lx <= 0 || c->ly <= 0 || c->lz <= 0) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_add_label: bad size");
    const long long N = (long long)c->lx * c->ly * c->lz;
    if (N >= (1LL << 31)) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_add_label: box too large");
    // the compact layout of a tiled box is planned on the host, so the box comes back once
    std::vector<int8_t> nature((size_t)N);
    const int rc = lbgpu_geometry(b->device, label, c->lx, c->ly, c->lz, params, nature.data());
    if (rc) return rc;   // the reference's message is in lbgpu_last_error(NULL, ...)
    return lbgpu_batch_add(b, c, nature.data(), id);
}

int lbgpu_batch_add(lbgpu_batch *b, const lbgpu_cell *c, const int8_t *nature, int *id)
{
    TraceRange trace_("lbgpu_batch_add");
    if (!b || !c || !nature || !id) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_add: null argument");
    if (c->lx <= 0 || c->ly <= 0 || c->lz <= 0) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_add: bad size");
    if (!(c->relaxation_time > 0.5)) return bfail(LBGPU_ERR_INVALID, "relaxation_time must be > 0.5");
    const lbgpu_tracer &t = c->tracer;
    const bool tracer = t.Db != 0.0;
    if (tracer) {   // drop_tracers.f90:88-89, module_moment_propagation.f90:41-79
        if (!(t.Db > EPS)) return bfail(LBGPU_ERR_INVALID, "The diffusion coefficient (tracer_Db in input file) is invalid");
        if (t.ka < -EPS) return bfail(LBGPU_ERR_INVALID, "I detected tracer%ka to be <0");
        if (t.kd < -EPS) return bfail(LBGPU_ERR_INVALID, "I detected tracer%kd to be <0");
        if (std::fabs(t.Ds) > EPS) return bfail(LBGPU_ERR_UNSUPPORTED, "Tracers you defined have non-zero surface diffusion coefficient");
        if (std::fabs(t.z) > EPS) return bfail(LBGPU_ERR_UNSUPPORTED, "charged tracers are not implemented");
    }
    const long long N = (long long)c->lx * c->ly * c->lz;
    if ((unsigned long long)Q * N >= (1ULL << 32)) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_add: box too large");
    const bool ads = tracer && tracer_ads(t);
    for (long long i = 0; i < N; ++i)
        if (nature[i] != 0 && nature[i] != 1) return bfail(LBGPU_ERR_INVALID, "nature must be 0 or 1");
    Slot sl;
    sl.active = true;
    sl.tracer = tracer;
    sl.smem = batch_smem_flow((int)N) <= b->smem_max && (!tracer || batch_smem_mp((int)N, ads) <= b->smem_max);
    // tiled boxes: fluid-only layout (compact.cuh) built from the geometry on the host
    std::vector<uint2> tab;
    std::vector<uint32_t> pos;
    int nw = 0, xbits = 0, ybits = 0;
    const bool compact = !sl.smem;
    if (compact && !build_compact_tables(c->lx, c->ly, c->lz, nature, tab, pos, nw, xbits, ybits))
        return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_add: box shape beyond the packed-position limits");
    if (compact && pos.empty()) return bfail(LBGPU_ERR_INVALID, "All nodes are solid: no fluid, no fluid dynamics!");
    const long long units = compact ? (long long)pos.size() : N;
    // LBGPU_BATCH_SLAB=0: tiled boxes take node tiles in the tracer phase too (same bits)
    const char *slab_env = std::getenv("LBGPU_BATCH_SLAB");
    const bool slab_ok = !(slab_env && std::string(slab_env) == "0");
    const int nslab = compact && tracer && slab_ok ? batch_slab_tiles(c->lx, c->ly, c->lz) : 0;
    const int ntacc = std::max((int)((units + BATCH_BLOCK - 1) / BATCH_BLOCK), nslab);
    sl.slab_live.clear();
    if (nslab) {   // slab tile k: column tile k % nxy (MPS_TX x MPS_TY), planes [zc (k / nxy), + zc)
        const int tx = (c->lx + MPS_TX - 1) / MPS_TX, nxy = tx * ((c->ly + MPS_TY - 1) / MPS_TY);
        for (int k = 0; k < nslab; ++k) {
            const int t = k % nxy, x0 = (t % tx) * MPS_TX, y0 = (t / tx) * MPS_TY, z0 = (k / nxy) * BATCH_SLAB_ZC;
            bool fluid = false;
            for (int z = z0; z < std::min(z0 + BATCH_SLAB_ZC, c->lz) && !fluid; ++z)
                for (int y = y0; y < std::min(y0 + MPS_TY, c->ly) && !fluid; ++y)
                    for (int x = x0; x < std::min(x0 + MPS_TX, c->lx); ++x)
                        if (nature[(size_t)x + (size_t)c->lx * ((size_t)y + (size_t)c->ly * z)] == 0) {
                            fluid = true;
                            break;
                        }
            if (fluid) sl.slab_live.push_back(k);
        }
    }
    const Layout L = layout(N, units, (long long)tab.size(), ntacc, compact, tracer, ads);
    if (b->used + L.total > b->budget)
        return bfail(LBGPU_ERR_OOM, "lbgpu_batch_add: box needs " + std::to_string(L.total >> 20) +
                                        " MiB beyond the batch memory budget");
    cudaStream_t s = b->stream;
    sl.bytes = L.total;
    sl.ntile = ntacc;
    LBB_CK(cudaMallocAsync(&sl.mem, L.total, s));
    char *base = static_cast<char *>(sl.mem);
    BatchInst &d = sl.d;
    std::memset(&d, 0, sizeof(d));
    d.lx = c->lx;
    d.ly = c->ly;
    d.lz = c->lz;
    d.N = (int)N;
    d.phase = BATCH_FLOW;
    d.ads = ads ? 1 : 0;
    d.zc = nslab ? BATCH_SLAB_ZC : 0;
    d.ntacc = ntacc;
    fill_consts(d, *c);
    d.g = reinterpret_cast<float *>(base + L.g);
    uint32_t *mask = reinterpret_cast<uint32_t *>(base + L.mask);
    d.mask = mask;
    d.uprev = reinterpret_cast<float4 *>(base + L.uprev);
    int8_t *d_nature = reinterpret_cast<int8_t *>(base + L.nature);
    if (compact) {
        d.compact = 1;
        d.Nf = (unsigned)units;
        d.nw = nw;
        d.xbits = xbits;
        d.ybits = ybits;
        d.cpos = reinterpret_cast<uint32_t *>(base + L.cpos);
        d.cmask = reinterpret_cast<uint32_t *>(base + L.cmask);
        d.rowtab = reinterpret_cast<uint2 *>(base + L.rowtab);
    }
    if (tracer) {
        d.V = reinterpret_cast<float4 *>(base + L.V);
        d.P[0] = reinterpret_cast<float4 *>(base + L.P0);
        d.P[1] = reinterpret_cast<float4 *>(base + L.P1);
        if (ads) {
            d.A[0] = reinterpret_cast<float4 *>(base + L.A0);
            d.A[1] = reinterpret_cast<float4 *>(base + L.A1);
        }
        d.aux = reinterpret_cast<float4 *>(base + L.aux);
        d.tacc = reinterpret_cast<double *>(base + L.tacc);
    }
    LBB_CK(cudaMemsetAsync(sl.mem, 0, L.total, s));   // rest state rho = rho0, j = 0; P = A = V = 0
    LBB_CK(cudaMemcpyAsync(d_nature, nature, N, cudaMemcpyHostToDevice, s));
    LBB_CK(launch_node_flags(d_nature, mask, c->lx, c->ly, c->lz, s));
    if (compact) {
        LBB_CK(cudaMemcpyAsync((void *)d.cpos, pos.data(), sizeof(uint32_t) * pos.size(), cudaMemcpyHostToDevice, s));
        LBB_CK(cudaMemcpyAsync((void *)d.rowtab, tab.data(), sizeof(uint2) * tab.size(), cudaMemcpyHostToDevice, s));
        FlowArgs32 fa;
        std::memset(&fa, 0, sizeof(fa));
        fa.mask = mask;
        fa.Nf = d.Nf;
        fa.cpos = d.cpos;
        fa.lx = d.lx;
        fa.ly = d.ly;
        fa.xbits = xbits;
        fa.ybits = ybits;
        LBB_CK(launch_compact_mask(fa, const_cast<uint32_t *>(d.cmask), s));
    }
    LBB_CK(cudaMemsetAsync(b->d_counts, 0, 4 * sizeof(unsigned long long), s));
    LBB_CK(launch_count_nodes(mask, N, b->d_counts, s));
    unsigned long long counts[4];
    LBB_CK(cudaMemcpyAsync(counts, b->d_counts, sizeof(counts), cudaMemcpyDeviceToHost, s));
    LBB_CK(cudaStreamSynchronize(s));   // the caller may reuse nature; host tables go out of scope
    if (!counts[0]) {
        cudaFreeAsync(sl.mem, s);
        return bfail(LBGPU_ERR_INVALID, "All nodes are solid: no fluid, no fluid dynamics!");
    }
    sl.fluid = (long long)counts[0];
    if (tracer) {   // module_moment_propagation.f90:97
        const double K = std::fabs(t.kd) <= EPS ? 0.0 : t.ka / t.kd;
        d.bw = (float)(1.0 / ((double)counts[0] + K * (double)counts[2]));
    }
    int k = 0;
    while (k < (int)b->slots.size() && b->slots[k].active) ++k;
    if (k == (int)b->slots.size()) b->slots.push_back(sl);
    else b->slots[k] = sl;
    b->used += L.total;
    b->dirty = true;
    *id = k;
    return LBGPU_OK;
}

int lbgpu_batch_remove(lbgpu_batch *b, int id)
{
    if (!valid_slot(b, id)) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_remove: no such box");
    Slot &sl = b->slots[id];
    LBB_CK(cudaFreeAsync(sl.mem, b->stream));
    b->used -= sl.bytes;
    sl = Slot();
    b->dirty = true;
    return LBGPU_OK;
}

int lbgpu_batch_steps(lbgpu_batch *b, int nsteps, int check, float *du)
{
    TraceRange trace_("lbgpu_batch_steps");
    if (!b || nsteps < 0 || (nsteps & 1)) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_steps: nsteps must be even and >= 0");
    int rc = rebuild(b);
    if (rc) return rc;
    if (b->desc_slot.empty() || nsteps == 0) return LBGPU_OK;
    if ((rc = run_steps(b, nsteps, check != 0))) return rc;
    if (check && du) {
        std::vector<unsigned> h(b->desc_slot.size());
        LBB_CK(cudaMemcpyAsync(h.data(), b->d_du, sizeof(unsigned) * h.size(), cudaMemcpyDeviceToHost, b->stream));
        LBB_CK(cudaStreamSynchronize(b->stream));
        for (size_t i = 0; i < h.size(); ++i) {
            float f;
            std::memcpy(&f, &h[i], sizeof(f));
            du[b->desc_slot[i]] = f;
        }
        return LBGPU_OK;
    }
    LBB_CK(cudaStreamSynchronize(b->stream));
    return LBGPU_OK;
}

int lbgpu_batch_time_steps(lbgpu_batch *b, int nsteps, float *ms)
{
    if (!b || !ms || nsteps < 0 || (nsteps & 1)) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_time_steps: bad argument");
    int rc = rebuild(b);
    if (rc) return rc;
    const bool work = !b->desc_slot.empty() && nsteps > 0;
    if ((rc = tune_aa(b)) || (rc = tune_smem(b))) return rc;             // outside the timed region
    if (work && (rc = call_graphs(b, nsteps, false, false))) return rc;
    LBB_CK(cudaEventRecord(b->ev0, b->stream));
    if (work && (rc = run_steps(b, nsteps, false))) return rc;
    LBB_CK(cudaEventRecord(b->ev1, b->stream));
    LBB_CK(cudaEventSynchronize(b->ev1));
    LBB_CK(cudaEventElapsedTime(ms, b->ev0, b->ev1));
    return LBGPU_OK;
}

int lbgpu_batch_get_tuning(lbgpu_batch *b, lbgpu_batch_tuning *out)
{
    if (!b || !out) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_get_tuning: null argument");
    std::memset(out, 0, sizeof(*out));
    out->tuned = b->aa_tuned ? 1 : 0;
    for (int k = 0; k < 2; ++k) {
        out->aa_work_list[k] = b->aa_list[k];
        out->aa_min_blocks[k] = b->aa_minb[k];
        out->aa_tiles_per_claim[k] = b->aa_tpc[k];
        out->aa_ms[k] = b->aa_ms[k];
    }
    out->smem_threads = b->smem_threads;
    out->steps_per_graph = b->steps_per_graph;
    out->tiled_fluid_nodes = b->tuned_fluid;
    return LBGPU_OK;
}

int lbgpu_batch_moments(lbgpu_batch *b, int id, double *rho, double *jx, double *jy, double *jz)
{
    if (!valid_slot(b, id) || !rho || !jx || !jy || !jz)
        return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_moments: bad argument");
    int rc = rebuild(b);
    if (rc) return rc;
    const int desc = desc_of(b, id);
    const BatchInst &d = b->slots[id].d;
    const int N = d.N;
    cudaStream_t s = b->stream;
    double *tmp = nullptr;
    LBB_CK(cudaMallocAsync((void **)&tmp, sizeof(double) * 4 * (size_t)N, s));
    if (d.compact) LBB_CK(cudaMemsetAsync(tmp, 0, sizeof(double) * 4 * (size_t)N, s));   // solid nodes: zeros
    LBB_CK(launch_batch_moments(b->d_insts, desc, batch_units(d), tmp, tmp + N, tmp + 2 * (size_t)N,
                                tmp + 3 * (size_t)N, s));
    double *out[4] = {rho, jx, jy, jz};
    for (int q = 0; q < 4; ++q)
        LBB_CK(cudaMemcpyAsync(out[q], tmp + q * (size_t)N, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    LBB_CK(cudaFreeAsync(tmp, s));
    LBB_CK(cudaStreamSynchronize(s));
    return LBGPU_OK;
}

int lbgpu_batch_mp_start(lbgpu_batch *b, int id)
{
    TraceRange trace_("lbgpu_batch_mp_start");
    if (!valid_slot(b, id)) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_mp_start: no such box");
    Slot &sl = b->slots[id];
    if (!sl.tracer) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_mp_start: the box has no tracer (tracer.Db = 0)");
    if (sl.d.phase != BATCH_FLOW) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_mp_start: tracer phase already started");
    int rc = rebuild(b);
    if (rc) return rc;
    cudaStream_t s = b->stream;
    LBB_CK(launch_batch_mp_start(b->d_insts, desc_of(b, id), batch_units(sl.d), s));
    unsigned st = 0;
    LBB_CK(cudaMemcpyAsync(&st, sl.d.tacc + (size_t)sl.ntile * BATCH_TACC, sizeof(st), cudaMemcpyDeviceToHost, s));
    LBB_CK(cudaStreamSynchronize(s));
    if (st & LBGPU_ERR_FRACTION)   // module_moment_propagation.f90:249-257
        return bfail(LBGPU_ERR_FRACTION, "remaining fraction below epsilon: reduce the adsorption rate");
    sl.d.phase = BATCH_MP;
    sl.mp_steps = 0;
    b->dirty = true;
    return LBGPU_OK;
}

int lbgpu_batch_mp_get(lbgpu_batch *b, int id, double vacf0[3], double vacf_sum[3],
                       double vacf_last[3], int *steps)
{
    if (!valid_slot(b, id)) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_mp_get: no such box");
    const Slot &sl = b->slots[id];
    if (sl.d.phase != BATCH_MP) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_mp_get: no tracer phase");
    std::vector<double> h((size_t)sl.ntile * BATCH_TACC);
    LBB_CK(cudaMemcpyAsync(h.data(), sl.d.tacc, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, b->stream));
    LBB_CK(cudaStreamSynchronize(b->stream));
    double *outs[3] = {vacf0, vacf_sum, vacf_last};
    for (int q = 0; q < 3; ++q) {
        if (!outs[q]) continue;
        for (int d = 0; d < 3; ++d) {
            double acc = 0.0;
            for (int t = 0; t < sl.ntile; ++t) acc += h[(size_t)t * BATCH_TACC + 3 * q + d];
            outs[q][d] = acc;
        }
    }
    if (steps) *steps = sl.mp_steps;
    return LBGPU_OK;
}

int lbgpu_batch_mp_fields(lbgpu_batch *b, int id, double *P, double *P_ads)
{
    if (!valid_slot(b, id)) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_mp_fields: no such box");
    const Slot &sl = b->slots[id];
    if (sl.d.phase != BATCH_MP) return bfail(LBGPU_ERR_INVALID, "lbgpu_batch_mp_fields: no tracer phase");
    const size_t N = (size_t)sl.d.N;
    std::vector<float4> f(N);
    double *outs[2] = {P, P_ads};
    for (int q = 0; q < 2; ++q) {
        if (!outs[q]) continue;
        const float4 *src = q == 0 ? sl.d.P[0] : sl.d.A[0];   // a call runs an even number of steps
        if (!src) {
            std::memset(outs[q], 0, sizeof(double) * 3 * N);
            continue;
        }
        LBB_CK(cudaMemcpyAsync(f.data(), src, sizeof(float4) * N, cudaMemcpyDeviceToHost, b->stream));
        LBB_CK(cudaStreamSynchronize(b->stream));
        for (size_t i = 0; i < N; ++i) {
            outs[q][3 * i] = f[i].x;
            outs[q][3 * i + 1] = f[i].y;
            outs[q][3 * i + 2] = f[i].z;
        }
    }
    return LBGPU_OK;
}

int lbgpu_batch_info(lbgpu_batch *b, int *active, long long *fluid_nodes, int *smem_boxes,
                     size_t *bytes_used)
{
    if (!b) return LBGPU_ERR_INVALID;
    int a = 0, sm = 0;
    long long f = 0;
    for (auto &sl : b->slots)
        if (sl.active) {
            ++a;
            f += sl.fluid;
            sm += sl.smem;
        }
    if (active) *active = a;
    if (fluid_nodes) *fluid_nodes = f;
    if (smem_boxes) *smem_boxes = sm;
    if (bytes_used) *bytes_used = b->used;
    return LBGPU_OK;
}

int lbgpu_serve(lbgpu_batch *b, const lbgpu_request *req, int n, double du_tol, int check_every,
                lbgpu_request_result *out)
{
    TraceRange trace_("lbgpu_serve");
    if (!b || n < 0 || (n > 0 && (!req || !out)) || check_every <= 0 || (check_every & 1))
        return bfail(LBGPU_ERR_INVALID, "lbgpu_serve: bad argument (check_every must be even and > 0)");
    for (auto &sl : b->slots)
        if (sl.active) return bfail(LBGPU_ERR_INVALID, "lbgpu_serve: the batch must be empty");
    for (int i = 0; i < n; ++i)
        if (req[i].mp_steps > 0 && !(req[i].cell.tracer.Db > 0.0))
            return bfail(LBGPU_ERR_INVALID, "lbgpu_serve: tracer steps requested without a tracer");
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return req[x].arrival < req[y].arrival; });
    for (int i = 0; i < n; ++i) {
        std::memset(&out[i], 0, sizeof(out[i]));
        out[i].admitted = out[i].finished = -1.0;
    }
    std::vector<int> slot_req;   // slot -> request index (-1 when free)
    std::vector<int> checks(n, 0);
    std::vector<int> phase_before;
    std::vector<float> du;
    const double t0 = now_s();
    int next = 0, done = 0, rc;
    auto finish = [&](int k, int r, double t) -> int {
        out[r].finished = t;
        slot_req[k] = -1;
        ++done;
        return lbgpu_batch_remove(b, k);
    };
    while (done < n) {
        double t = now_s() - t0;
        // admission: in arrival order, while the head request has arrived and fits
        while (next < n && req[order[next]].arrival <= t) {
            const int r = order[next];
            const lbgpu_request &q = req[r];
            const size_t need = lbgpu_batch_footprint(&q.cell);
            if (need == 0 || need > b->budget) {   // can never fit: rejected, the queue moves on
                out[r].status = need == 0 ? LBGPU_ERR_INVALID : LBGPU_ERR_OOM;
                ++next;
                ++done;
                continue;
            }
            if (b->used + need > b->budget) break;
            int id = -1;
            rc = lbgpu_batch_add(b, &q.cell, q.nature, &id);
            if (rc == LBGPU_ERR_INVALID || rc == LBGPU_ERR_UNSUPPORTED) {
                out[r].status = rc;
                ++next;
                ++done;
                continue;
            }
            if (rc) return rc;
            if ((int)slot_req.size() <= id) slot_req.resize(id + 1, -1);
            slot_req[id] = r;
            out[r].admitted = now_s() - t0;
            out[r].fluid_nodes = b->slots[id].fluid;
            ++next;
        }
        bool any = false;
        for (auto &sl : b->slots) any |= sl.active;
        if (!any) {
            if (next >= n) break;
            const double wait = req[order[next]].arrival - (now_s() - t0);
            if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
            continue;
        }
        phase_before.assign(b->slots.size(), -1);
        for (size_t k = 0; k < b->slots.size(); ++k)
            if (b->slots[k].active) phase_before[k] = b->slots[k].d.phase;
        du.assign(b->slots.size(), 0.0f);
        if ((rc = lbgpu_batch_steps(b, check_every, 1, du.data()))) return rc;
        t = now_s() - t0;
        for (size_t k = 0; k < b->slots.size(); ++k) {
            if (phase_before[k] < 0) continue;
            const int r = slot_req[k];
            const lbgpu_request &q = req[r];
            if (phase_before[k] == BATCH_MP) {
                const int target = (q.mp_steps + check_every - 1) / check_every * check_every;
                if (b->slots[k].mp_steps >= target) {
                    if ((rc = lbgpu_batch_mp_get(b, (int)k, out[r].vacf0, out[r].vacf_sum, nullptr, &out[r].mp_steps)))
                        return rc;
                    if ((rc = finish((int)k, r, t))) return rc;
                }
                continue;
            }
            out[r].steps += check_every;
            checks[r] += 1;
            const bool bad = !std::isfinite(du[k]);
            const bool conv = checks[r] >= 2 && du[k] < du_tol;
            const bool cap = q.max_steps > 0 && out[r].steps >= q.max_steps;
            if (!(conv || cap || bad)) continue;
            out[r].converged = conv ? 1 : 0;
            if (!conv) out[r].status |= LBGPU_ERR_STEP_CAP;   // flagged; its tracer steps still run
            if (bad) {
                out[r].status = LBGPU_ERR_NONFINITE;
                if ((rc = finish((int)k, r, t))) return rc;
                continue;
            }
            if (q.out_density && q.out_jx && q.out_jy && q.out_jz &&
                (rc = lbgpu_batch_moments(b, (int)k, q.out_density, q.out_jx, q.out_jy, q.out_jz)))
                return rc;
            if (q.mp_steps > 0) {
                rc = lbgpu_batch_mp_start(b, (int)k);
                if (rc == LBGPU_OK) continue;
                if (rc != LBGPU_ERR_FRACTION) return rc;
                out[r].status |= rc;
            }
            if ((rc = finish((int)k, r, now_s() - t0))) return rc;
        }
    }
    return LBGPU_OK;
}

}  // extern "C"
