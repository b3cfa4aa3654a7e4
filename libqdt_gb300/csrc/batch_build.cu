// The batch build's kernels that evaluate predicates -- the per-height
// merges, their persistent form, the shared-memory cells and the extraction's
// orientation test -- with their launchers (batch_kernels.hpp). Like
// k_build.cu, this file is compiled twice: here with QDTG_WIDE_EXACT 0
// (qdtg::narrow, run on every call) and from batch_build_wide.cu with the
// widest exact tier (qdtg::wide, run again on the rare batch whose
// predicates needed it).
//
// The merges follow the reference builder (builder.hxx:177-301) through the
// shared builder of builder.cuh; what is specific to the batch is the
// addressing of a node by (set, depth, index) through per-height entry
// lists, and the persistent form's done flags.
#ifndef QDTG_BUILD_VARIANT
#define QDTG_WIDE_EXACT 0
#define QDTG_BUILD_VARIANT narrow
#endif

#include "batch_kernels.hpp"
#include "builder.cuh"
#include "common.cuh"
#include "predicates.cuh"

namespace qdtg {
namespace QDTG_BUILD_VARIANT {

namespace {

// the sleeps a persistent-build warp waits for a child before it reports a
// fault
constexpr long long kPersistSpin = 1ll << 22;

// All nodes of one height (the levels below them) in every participating
// set. Nodes of equal height have sizes within a factor of two, so the
// merges of a launch are alike, whatever the sizes of their sets; a node's
// children have smaller heights and were built by earlier launches. A node
// of height h lies at depth D - h (D the set's split depth) or, when it is a
// smaller sibling, at D - h - 1: the launch runs over entries (set, depth)
// with 2^depth slots each (entry e covers slots [eoff[e], eoff[e + 1])) and
// skips the slots whose node has another height. The single-set
// k_build_level is the same body with depth-synchronous launches (there all
// nodes of a depth are alike).
// One node slot of height h (flat index into the height's entries): a
// leaf, or the merge of its children. PERSIST: 0 for the launch per height;
// in the persistent form, where the children may still be in flight on
// other warps, 1 waits for their done flags (bounded) here and 2 has had
// them waited for by its caller; both set the node's own flag.
template <bool WARP, bool LEAF, int PERSIST>
__device__ __forceinline__ void bbuild_node(Rec* __restrict__ R, int nrec, const double2* __restrict__ V,
    NodeOut* __restrict__ nodes, const uint32_t* __restrict__ noff, const uint32_t* __restrict__ ent,
    const uint32_t* __restrict__ eoff, int nent, const uint32_t* __restrict__ u_off, int h, long long flat, int lane,
    DevStatus* st, int count, uint32_t* __restrict__ done)
{
    const uint32_t  e = find_set(eoff, nent, (uint32_t)flat);
    const uint32_t  s = ent[e] >> 5;
    const int       d = (int)(ent[e] & 31u);
    const long long k = flat - eoff[e];
    const int       base = (int)u_off[s], ms = (int)(u_off[s + 1] - u_off[s]);
    int             lo, hi;
    if (!node_range(ms, d, k, lo, hi) || subtree_levels(hi - lo) != h) return;
    lo += base;
    hi += base;
    NodeOut* const out = nodes + noff[s];   // heap order: (1 << depth) + index
    const int      n = hi - lo;
    Builder        B{ R, nrec, st,
        pred_stage(st, (LEAF || n <= 3) ? kStageLeaf : (WARP ? kStageWarp : kStageThread), count), -1, -1, false };
    NodeOut        o;
    // height 0 is all leaves, the other heights all merges: two kernels, so
    // that neither carries the other's code
    o.le2 = o.re2 = -1;
    o.pad0 = o.pad1 = 0;
    if (LEAF || n <= 3)
    {
        if (!LEAF || lane != 0) return;
        B.leaf(lo, hi, V, o.le, o.re);
        if (d > 0 && !B.bad) extremes_by_walk(B, o.le, o.re, d & 1, 8, o.le2, o.re2);
    }
    else
    {
        if (PERSIST == 1)
        {
            // both children done: their node records and every record edit
            // below them (each done flag was set after a device-wide fence)
            bool ok = true;
            if (!WARP || lane == 0)
            {
                const volatile uint32_t* f = done + noff[s] + (2ll << d) + 2 * k;
                for (long long i = 0; !(f[0] && f[1]); ++i)
                {
                    if (i > kPersistSpin || (*(volatile unsigned*)&st->flags & kFatal))
                    {
                        ok = false;
                        break;
                    }
                    __nanosleep(64);
                }
                if (!ok) atomicOr(&st->flags, ST_GUARD);
            }
            if (WARP) ok = __shfl_sync(0xffffffffu, (int)ok, 0) != 0;
            if (!ok) return;
            __threadfence();
        }
        const NodeOut L = out[(2ll << d) + 2 * k], Rn = out[(2ll << d) + 2 * k + 1];
        if ((L.fhead >= 0 && (L.ftail < 3 * lo || L.ftail >= 3 * hi)) ||
            (Rn.fhead >= 0 && (Rn.ftail < 3 * lo || Rn.ftail >= 3 * hi)))
        {
            if (lane == 0) B.fail(ST_BAD_INDEX);
            return;
        }
        if (L.fhead >= 0)
        {
            B.fhead = L.fhead;
            if (Rn.fhead >= 0)
            {
                if (lane == 0) R[L.ftail].link = Rn.fhead;
                B.ftail = Rn.ftail;
            }
            else
                B.ftail = L.ftail;
        }
        else
        {
            B.fhead = Rn.fhead;
            B.ftail = Rn.ftail;
        }
        const int lim = 8 * n + 64;
        const int g = (d - 1) & 1;   // the parent's frame
        int       rl = 0, rr = 0;
        NodeOut*      self = &out[(1ll << d) + k];
        volatile int* first = nullptr;
        if (d > 0 && lane == 0)
        {
            extremes_before_merge(R, nrec, st, &out[(2ll << d) + 2 * k], &out[(2ll << d) + 2 * k + 1], self, g);
            first = lower_tangent_slot(self);
        }
        if (WARP) warp_merge(B, L.le, L.re, Rn.le, Rn.re, lim, rl, rr, first);
        else B.merge(L.le, L.re, Rn.le, Rn.re, lim, rl, rr, first);
        if (lane != 0) return;
        o.le2 = rl;
        o.re2 = rr;
        if (d > 0 && !B.bad)
        {
            const int2 x = extremes_after_merge(R, nrec, st, B.basel_last, self, &out[(2ll << d) + 2 * k],
                &out[(2ll << d) + 2 * k + 1], g, n + 8);
            rl = x.x;
            rr = x.y;
        }
        o.le = rl;
        o.re = rr;
    }
    B.settle_tail();
    o.fhead = B.fhead;
    o.ftail = B.ftail;
    out[(1ll << d) + k] = o;
    if (PERSIST)
    {
        __threadfence();   // the node and its edits before its flag
        *(volatile uint32_t*)(done + noff[s] + (1ll << d) + k) = 1u;
    }
}

template <bool WARP, bool LEAF>
__global__ void QDTG_BUILD_BOUNDS(WARP) k_bbuild_height(Rec* __restrict__ R, int nrec,
    const double2* __restrict__ V, NodeOut* __restrict__ nodes, const uint32_t* __restrict__ noff,
    const uint32_t* __restrict__ ent, const uint32_t* __restrict__ eoff, int nent, const uint32_t* __restrict__ u_off,
    int h, DevStatus* st, int count)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long flat = WARP ? (g >> 5) : g;
    const int       lane = WARP ? (int)(threadIdx.x & 31) : 0;
    if (flat >= (long long)eoff[nent]) return;
    unsigned flags = *(volatile unsigned*)&st->flags;
    if (WARP) flags = __shfl_sync(0xffffffffu, flags, 0);
    if (flags & kFatal) return;
    bbuild_node<WARP, LEAF, 0>(R, nrec, V, nodes, noff, ent, eoff, nent, u_off, h, flat, lane, st, count,
        nullptr);
}

// The persistent form of the same build: one launch of resident warps that
// take work units from a counter, heights in increasing order (a unit is 32
// node slots, one a lane, at the thread heights, and one slot at the warp
// heights). A merge waits for its two children's done flags, which every
// warp sets after a device-wide fence; units are handed out in order and
// children have smaller heights, so the unit a merge waits for is already in
// some resident warp's hands, and every wait ends. Each wait is bounded
// (kPersistSpin sleeps); one that runs out sets ST_GUARD.
// The three forms of a node in the persistent kernel, each out of line so
// that each gets its own register allocation.
__device__ __noinline__ void persist_warp_node(Rec* __restrict__ R, int nrec, const double2* __restrict__ V,
    NodeOut* __restrict__ nodes, const uint32_t* __restrict__ noff, const uint32_t* __restrict__ en,
    const uint32_t* __restrict__ eo, int ne, const uint32_t* __restrict__ u_off, int h, long long flat, int lane,
    DevStatus* st, int count, uint32_t* __restrict__ done)
{
    bbuild_node<true, false, 1>(R, nrec, V, nodes, noff, en, eo, ne, u_off, h, flat, lane, st, count, done);
}

__device__ __noinline__ void persist_leaf(Rec* __restrict__ R, int nrec, const double2* __restrict__ V,
    NodeOut* __restrict__ nodes, const uint32_t* __restrict__ noff, const uint32_t* __restrict__ en,
    const uint32_t* __restrict__ eo, int ne, const uint32_t* __restrict__ u_off, long long flat, DevStatus* st,
    int count, uint32_t* __restrict__ done)
{
    bbuild_node<false, true, 2>(R, nrec, V, nodes, noff, en, eo, ne, u_off, 0, flat, 0, st, count, done);
}

__device__ __noinline__ void persist_thread_node(Rec* __restrict__ R, int nrec, const double2* __restrict__ V,
    NodeOut* __restrict__ nodes, const uint32_t* __restrict__ noff, const uint32_t* __restrict__ en,
    const uint32_t* __restrict__ eo, int ne, const uint32_t* __restrict__ u_off, int h, long long flat,
    DevStatus* st, int count, uint32_t* __restrict__ done)
{
    bbuild_node<false, false, 2>(R, nrec, V, nodes, noff, en, eo, ne, u_off, h, flat, 0, st, count, done);
}

__global__ void __maxnreg__(168) k_bbuild_persist(Rec* __restrict__ R, int nrec, const double2* __restrict__ V,
    NodeOut* __restrict__ nodes, const uint32_t* __restrict__ noff, const uint32_t* __restrict__ ents,
    const uint32_t* __restrict__ eoffs, const uint32_t* __restrict__ u_off, uint32_t* __restrict__ counter,
    uint32_t* __restrict__ done, DevStatus* st, int count, const PersistPlan* __restrict__ plan)
{
    const unsigned FULL = 0xffffffffu;
    const int      lane = threadIdx.x & 31;
    const int      nh = plan->nh;
    const uint32_t total = plan->unit_off[nh];
    for (;;)
    {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(counter, 1u);
        u = __shfl_sync(FULL, u, 0);
        if (u >= total) return;
        if (__shfl_sync(FULL, *(volatile unsigned*)&st->flags, 0) & kFatal) return;
        int h = 0;
        while (h + 1 < nh && plan->unit_off[h + 1] <= u) ++h;
        const uint32_t  local = u - plan->unit_off[h];
        const uint32_t* en = ents + plan->ent0[h];
        const uint32_t* eo = eoffs + plan->eoff0[h];
        const int       ne = plan->nent[h];
        const long long slots = eo[ne];
        if (plan->warp[h])
            persist_warp_node(R, nrec, V, nodes, noff, en, eo, ne, u_off, h, (long long)local, lane, st, count, done);
        else
        {
            const long long flat = (long long)local * 32 + lane;
            if (h > 0)
            {
                // the whole warp waits until the children of all its lanes'
                // nodes are done, so that the lanes start their merges
                // together
                const volatile uint32_t* f = nullptr;
                if (flat < slots)
                {
                    const uint32_t e = find_set(eo, ne, (uint32_t)flat);
                    const uint32_t s = en[e] >> 5;
                    const int      d = (int)(en[e] & 31u);
                    const long long k = flat - eo[e];
                    int             lo, hi;
                    if (node_range((int)(u_off[s + 1] - u_off[s]), d, k, lo, hi) && subtree_levels(hi - lo) == h)
                        f = done + noff[s] + (2ll << d) + 2 * k;
                }
                bool ok = true;
                for (long long i = 0;; ++i)
                {
                    if (__all_sync(FULL, !f || (f[0] && f[1]))) break;
                    const unsigned fl = __shfl_sync(FULL, lane == 0 ? *(volatile unsigned*)&st->flags : 0u, 0);
                    if (i > kPersistSpin || (fl & kFatal))
                    {
                        ok = false;
                        break;
                    }
                    __nanosleep(64);
                }
                if (!ok)
                {
                    if (lane == 0) atomicOr(&st->flags, ST_GUARD);
                    return;
                }
                __threadfence();
            }
            if (flat < slots)
            {
                if (h == 0) persist_leaf(R, nrec, V, nodes, noff, en, eo, ne, u_off, flat, st, count, done);
                else persist_thread_node(R, nrec, V, nodes, noff, en, eo, ne, u_off, h, flat, st, count, done);
            }
        }
        __syncwarp();
    }
}

// The cells of every set, one warp each: cell g belongs to the set s with
// cell_off[s] <= g < cell_off[s + 1] and is node g - cell_off[s] of the set's
// cell depth.
__global__ void __launch_bounds__(kCellBlockWarps * 32) k_bbuild_cells(Rec* __restrict__ R,
    const double2* __restrict__ V, NodeOut* __restrict__ nodes, const uint32_t* __restrict__ noff,
    const uint32_t* __restrict__ cell_off, int S, const uint32_t* __restrict__ u_off, int C, uint32_t ncells,
    DevStatus* st, int count)
{
    extern __shared__ __align__(16) char bcell_smem[];
    const int      w = threadIdx.x >> 5;
    const uint32_t g = blockIdx.x * (blockDim.x >> 5) + w;
    if (g >= ncells) return;
    const unsigned flags = __shfl_sync(0xffffffffu, *(volatile unsigned*)&st->flags, 0);
    if (flags & kFatal) return;
    const uint32_t  s = find_set(cell_off, S, g);
    const int       base = (int)u_off[s], ms = (int)(u_off[s + 1] - u_off[s]);
    const int       dc = cell_depth(ms, C);
    const long long k = (long long)(g - cell_off[s]);
    int             lo, hi;
    if (!node_range(ms, dc, k, lo, hi) || hi - lo > C) return;
    build_cell(bcell_smem + w * cell_smem_bytes(C), V, R, base + lo, base + hi, dc, st, pred_stage(st, kStageThread, count),
        nodes + noff[s] + (1ll << dc) + k);
}

// extraction; records of sets that were not built are skipped
__global__ void k_btri_mask(const Rec* __restrict__ R, int nrec, const uint32_t* __restrict__ useg,
    const uint8_t* __restrict__ skip, uint8_t* __restrict__ mask, DevStatus* st, int count)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nrec) return;
    if ((*(volatile unsigned*)&st->flags & kFatal) || skip[useg[k / 3]])
    {
        mask[k] = 0;
        return;
    }
    Builder B{ const_cast<Rec*>(R), nrec, st, pred_stage(st, kStageExtract, count), -1, -1, false };
    uint8_t mk = 0;
    if (R[k].org[0] >= 0)
    {
        for (int s = 0; s < 2; ++s)
        {
            const int e = 2 * k + s;
            const int f = B.lnext(e), g = B.lnext(f);
            if (B.lnext(g) != e) continue;
            if (e > f || e > g) continue;
            if (ccw(B.porg(e), B.porg(f), B.porg(g), B.pc)) mk |= (uint8_t)(1 << s);
        }
    }
    mask[k] = B.bad ? 0 : mk;
}

}  // namespace

void launch_bbuild_cells(const BatchBuildArgs& a, cudaStream_t s)
{
    const int warps = cell_block_warps(a.cell_points);
    const int smem = warps * cell_smem_bytes(a.cell_points);
    cudaFuncSetAttribute(k_bbuild_cells, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_bbuild_cells<<<(a.ncells + warps - 1) / warps, warps * 32, smem, s>>>(a.recs, a.V, a.nodes, a.noff,
        a.cell_off, a.S, a.u_off, a.cell_points, a.ncells, a.status, a.count);
}

void launch_bbuild_height(const BatchBuildArgs& a, int h, const uint32_t* en, const uint32_t* eo, int nent,
    long long slots, bool warp, cudaStream_t s)
{
    if (h == 0)
        k_bbuild_height<false, true><<<(unsigned)((slots + 127) / 128), 128, 0, s>>>(a.recs, a.nrec, a.V, a.nodes,
            a.noff, en, eo, nent, a.u_off, h, a.status, a.count);
    else if (warp)
        k_bbuild_height<true, false><<<(unsigned)((slots * 32 + 127) / 128), 128, 0, s>>>(a.recs, a.nrec, a.V,
            a.nodes, a.noff, en, eo, nent, a.u_off, h, a.status, a.count);
    else
        k_bbuild_height<false, false><<<(unsigned)((slots + 127) / 128), 128, 0, s>>>(a.recs, a.nrec, a.V, a.nodes,
            a.noff, en, eo, nent, a.u_off, h, a.status, a.count);
}

void launch_bbuild_persist(const BatchBuildArgs& a, const PersistPlan* plan, int grid, cudaStream_t s)
{
    k_bbuild_persist<<<(unsigned)grid, 128, 0, s>>>(a.recs, a.nrec, a.V, a.nodes, a.noff, a.ents, a.eoffs, a.u_off,
        a.counter, a.done, a.status, a.count, plan);
}

int persist_blocks_per_sm()
{
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_bbuild_persist, 128, 0) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    return per;
}

void launch_btri_mask(const BatchBuildArgs& a, cudaStream_t s)
{
    k_btri_mask<<<(unsigned)((a.nrec + 255) / 256), 256, 0, s>>>(a.recs, a.nrec, a.useg, a.skip, a.mask, a.status,
        a.count);
}

}  // namespace QDTG_BUILD_VARIANT
}  // namespace qdtg
