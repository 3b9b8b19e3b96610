// Window-staged fused PBR-block + CSR-remainder SpMM (sm_103a, FP32).
//
// A CTA owns a window of kWinRows consecutive rows at a time (for one column
// tile of 64 columns and one batch entry).  Graphs whose nodes are numbered
// by cluster (the reference's benchmark graphs, clustered / banded graphs,
// any graph after a locality ordering) put most nonzeros of those rows in
// the same kWinRows columns: the 2^20-node clustered R-MAT graph has 68.6 %
// of its nonzeros in the aligned 64 x 64 diagonal window.  Those X rows are
// staged once per window into shared memory by a bulk asynchronous copy
// (cp.async.bulk, completion on an mbarrier, kWinBufs windows in flight), so
// two thirds of the per-nonzero X-row reads come from shared memory instead
// of an L2 / HBM round trip; the rest are gathered from global memory in
// deep batches.
//
// Roles (kWinWarps + 1 warps per CTA):
//   * the producer warp draws work units from a global counter (so CTAs
//     balance dynamically); for each one it reads the window's stripe and row
//     pointers into shared memory and issues the bulk copy of the window's X
//     tile into the free buffer;
//   * the consumer warps take the unit's items (stripes of the window, or
//     pieces of heavy stripes) one at a time from a shared counter, so a
//     slow stripe does not hold the other warps back.  A warp decodes its
//     item's bitmask blocks and remainder entries into a list of (X-row
//     offset, row, value) entries in shared memory — entries whose column lies
//     in the staged window at the front, the others at the back — walks the
//     global entries in batches of kWinGather X-row gathers per half-warp,
//     then the window entries from shared memory, committing each row's sum
//     to its half-warp's tile, and writes every Y row once (no atomics, no
//     pre-zeroed Y).
//
// Half-warps: lanes 0-15 and 16-31 each cover the 64 columns of the tile
// with float4 lanes and take alternate entries; each has its own tile, and a
// row's result is tile0 + tile1 in that order, so results are deterministic.
// Heavy stripes (more than 2 x piece_work stored entries) are cut into
// pieces as in the stripe kernel (partial tiles in the workspace, reduced in
// piece order by the last piece to finish).
//
// Every wait on an mbarrier is bounded (about two seconds of SM clock); a
// wait that gives up records GL_ERR_TIMEOUT in the workspace's error word and
// the CTA stops drawing work.
#pragma once

#include "stripe_kernel.cuh"

namespace gl {

constexpr int kWinRows = 64;                      // rows per window = X rows staged per window
constexpr int kWinWarps = 8;                      // consumer warps
constexpr int kWinThreads = (kWinWarps + 1) * 32; // + the producer warp
constexpr int kWinCols = 64;                      // columns per tile: 16 lanes x float4
#ifndef GL_WIN_BUFS
#define GL_WIN_BUFS 3
#endif
#ifndef GL_WIN_PREFETCH_INFO
#define GL_WIN_PREFETCH_INFO 1
#endif
#ifndef GL_WIN_DYNAMIC_ITEMS
#define GL_WIN_DYNAMIC_ITEMS 1
#endif
#ifndef GL_WIN_MAXREG
#define GL_WIN_MAXREG 96
#endif
constexpr int kWinBufs = GL_WIN_BUFS;             // X windows in flight per CTA
constexpr int kWinList = 384;                     // list entries per warp (>= 2 x the largest piece_work)
constexpr int kWinMaxPieceWork = kWinList / 2;
constexpr int kWinInfo = 136;                     // per buffer: stripe pointers, heavy flags, row pointers
#ifndef GL_WIN_GATHER
#define GL_WIN_GATHER 8
#endif
constexpr int kWinGather = GL_WIN_GATHER;         // global X-row gathers in flight per half-warp
constexpr long long kWinTimeoutCycles = 4000000000LL;

// Shared memory of one CTA (dynamic; every region 16-byte aligned).
template <int BR>
struct WinSmem {
    static constexpr size_t xwin = 0;                                                   // [bufs][rows][64] f32
    static constexpr size_t xwin_bytes = (size_t)kWinBufs * kWinRows * kWinCols * 4;
    static constexpr size_t lists = xwin + xwin_bytes;                                  // [warps][list] uint2
    static constexpr size_t lists_bytes = (size_t)kWinWarps * kWinList * 8;
    static constexpr size_t tiles = lists + lists_bytes;                                // [warps][2][BR][64]
    static constexpr size_t tiles_bytes = (size_t)kWinWarps * 2 * BR * kWinCols * 4;
    static constexpr size_t rinfo = tiles + tiles_bytes;                                // [warps][16] i32
    static constexpr size_t rinfo_bytes = (size_t)kWinWarps * 16 * 4;
    static constexpr size_t winfo = rinfo + rinfo_bytes;                                // [bufs][kWinInfo] i32
    static constexpr size_t winfo_bytes = (size_t)kWinBufs * kWinInfo * 4;
    static constexpr size_t ctl = winfo + winfo_bytes;                                  // barriers, unit ids
    static constexpr size_t bytes = ctl + 128;
};

// ---- mbarrier / bulk-copy helpers (inline PTX) -----------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the phase with the given parity to complete; false after about
// kWinTimeoutCycles SM cycles.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kWinTimeoutCycles) return false;
    return true;
}
// Bulk copy global -> this CTA's shared memory; completes `bytes` of the
// mbarrier's transaction count.  dst, src 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// ---- list walking ------------------------------------------------------------
// One list entry: key = (float4 index of the X row << 3) | row-in-stripe and
// the value's bits.  The float4 index is column * K / 4 into X for global
// entries and column-in-window * 16 into the staged window for the others,
// so a lane's address is its base pointer + index (one shift, one
// multiply-add).
__device__ __forceinline__ uint32_t win_key(uint32_t f4, int r) { return (f4 << 3) | (uint32_t)r; }

__device__ __forceinline__ void win_fma(float4& acc, float v, const float4& x) {
    float2 a = make_float2(acc.x, acc.y), b = make_float2(acc.z, acc.w);
    const float2 vv = make_float2(v, v);
    a = __ffma2_rn(vv, make_float2(x.x, x.y), a);
    b = __ffma2_rn(vv, make_float2(x.z, x.w), b);
    acc = make_float4(a.x, a.y, b.x, b.y);
}

// Adds acc to row r of this half-warp's tile (ht: the lane's 4 columns of
// row 0); the first commit of a row stores instead of adding (touched: rows
// written so far).
__device__ __forceinline__ void win_commit(float* ht, int r, const float4& acc, uint32_t& touched) {
    float4* p = reinterpret_cast<float4*>(ht + r * kWinCols);
    if ((touched >> r) & 1u) {
        float4 o = *p;
        o.x += acc.x;
        o.y += acc.y;
        o.z += acc.z;
        o.w += acc.w;
        *p = o;
    } else {
        *p = acc;
        touched |= 1u << r;
    }
}

// One entry of a walk: a row change commits the running sum.
__device__ __forceinline__ void win_step(const uint2& en, const float4& x, float4& acc, int& cur, float* ht,
                                         uint32_t& touched) {
    const int r = (int)(en.x & 7u);
    if (r != cur) {
        if (cur >= 0) win_commit(ht, cur, acc, touched);
        acc = make_float4(0.f, 0.f, 0.f, 0.f);
        cur = r;
    }
    win_fma(acc, __uint_as_float(en.y), x);
}

// Walks entries [0, n) of a list segment: half-warp h takes entries h, h + 2,
// ...; NB X-row loads are issued before their FMAs (full batches without
// predicates, then one predicated tail).  base: the lane's float4 pointer
// into X (global) or into the staged window (shared).
template <int NB>
__device__ __forceinline__ void win_walk(const uint2* lst, int n, const float4* base, float* ht,
                                         uint32_t& touched, int h) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    int cur = -1;
    int e0 = 0;
    for (; e0 + 2 * NB <= n; e0 += 2 * NB) {
        uint2 en[NB];
        float4 x[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            en[q] = lst[e0 + 2 * q + h];
            x[q] = base[en[q].x >> 3];
        }
#pragma unroll
        for (int q = 0; q < NB; ++q) win_step(en[q], x[q], acc, cur, ht, touched);
    }
    if (e0 < n) {
        uint2 en[NB];
        float4 x[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const int e = e0 + 2 * q + h;
            if (e < n) {
                en[q] = lst[e];
                x[q] = base[en[q].x >> 3];
            }
        }
#pragma unroll
        for (int q = 0; q < NB; ++q)
            if (e0 + 2 * q + h < n) win_step(en[q], x[q], acc, cur, ht, touched);
    }
    if (cur >= 0) win_commit(ht, cur, acc, touched);
}

// Decodes one item (the blocks [b0, b1) and remainder entries [j0, j1) of
// a stripe; rstart[0..BR] in shared memory holds each row's first remainder
// entry, clamped to [j0, j1]) into the warp's list and accumulates it into
// the two half-warp tiles.  Returns false if the item has more entries than
// the list holds (the caller records an error).
template <int BR>
__device__ __forceinline__ bool win_unit(const StripeArgs<float>& a, int32_t b0, int32_t b1, int32_t j0, int32_t j1,
                                         const int32_t* rstart, int32_t xb, const float* xw, const float* Xg,
                                         uint2* lst, float* tile, uint32_t& touched, int lane) {
    constexpr int BC = BR;
    constexpr uint32_t ROWMASK = (BC >= 32) ? 0xffffffffu : ((1u << BC) - 1u);
    constexpr int NS = 2 * BR;   // row slots: [0, BR) window entries, [BR, 2 BR) global entries
    using RP = RowPack<NS>;
    const int h = lane >> 4;
    const uint32_t K4 = (uint32_t)(a.K >> 2);
    const int nrem = j1 - j0;
    // first two rounds of remainder entries in flight with the block metadata
    int32_t rcol[2];
    float rval[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int q = t * 32 + lane;
        rcol[t] = q < nrem ? a.rem_col[j0 + q] : 0;
        rval[t] = q < nrem ? a.rem_val[j0 + q] : 0.f;
    }
    int lpos = 0, gpos = 0;   // window entries from the front, global ones from the back
    bool ok = true;
    for (int32_t kc = b0; kc < b1; kc += 32) {
        const int nb = (b1 - kc) < 32 ? (b1 - kc) : 32;
        uint64_t code = 0;
        int32_t col0 = 0, off = 0;
        if (lane < nb) {
            code = static_cast<uint64_t>(a.codes[kc + lane]);
            col0 = a.coords[2 * (int64_t)(kc + lane) + 1];
            off = a.offsets[kc + lane];
        }
        const bool loc = lane < nb && (uint32_t)(col0 - xb) < (uint32_t)kWinRows;
        RP ex;
        ex.clear();
#pragma unroll
        for (int r = 0; r < BR; ++r) {
            const uint32_t c = __popc((uint32_t)(code >> (r * BC)) & ROWMASK);
            ex.set(r, loc ? c : 0u);
            ex.set(BR + r, loc ? 0u : c);
        }
        RP tot;
#pragma unroll
        for (int i = 0; i < RP::W; ++i) {
            const uint64_t mine = ex.w[i];
            uint64_t v = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            ex.w[i] = v - mine;
            tot.w[i] = __shfl_sync(0xffffffffu, v, 31);
        }
        int ltot = 0, gtot = 0;
#pragma unroll
        for (int r = 0; r < BR; ++r) {
            ltot += (int)tot.get(r);
            gtot += (int)tot.get(BR + r);
        }
        if (lpos + gpos + ltot + gtot + nrem > kWinList) {
            ok = false;
            break;
        }
        const int gbase = kWinList - gpos - gtot;
        const int npairs = nb * BR;
        for (int p0 = 0; p0 < npairs; p0 += 32) {
            const int p = p0 + lane;
            const int src = (p / BR) & 31;
            const int r = p % BR;
            const uint64_t bcode = __shfl_sync(0xffffffffu, code, src);
            const int32_t bcol0 = __shfl_sync(0xffffffffu, col0, src);
            const int32_t boff = __shfl_sync(0xffffffffu, off, src);
            const bool bloc = __shfl_sync(0xffffffffu, loc, src);
            const int slot = bloc ? r : BR + r;
            uint64_t bex = 0;
#pragma unroll
            for (int i = 0; i < RP::W; ++i) {
                const uint64_t w = __shfl_sync(0xffffffffu, ex.w[i], src);
                if ((slot >> 2) == i) bex = w;
            }
            const uint32_t rb = p < npairs ? (uint32_t)(bcode >> (r * BC)) & ROWMASK : 0u;
            if (rb) {
                const int32_t k0 = boff + __popcll(bcode & ((1ull << (r * BC)) - 1ull));
                const int within = (int)((bex >> (16 * (slot & 3))) & 0xffffu);
                int rowstart = 0;   // entries of the segment's earlier rows in this chunk
#pragma unroll
                for (int rr = 0; rr < BR - 1; ++rr)
                    rowstart += rr < r ? (int)(bloc ? tot.get(rr) : tot.get(BR + rr)) : 0;
                const int pos0 = (bloc ? lpos : gbase) + rowstart + within;
                // float4 index of column c of the block: global (bcol0 + c) * K4,
                // window (bcol0 - xb + c) * 16
                const uint32_t f0 = bloc ? (uint32_t)(bcol0 - xb) * 16u : (uint32_t)bcol0 * K4;
                const uint32_t fs = bloc ? 16u : K4;
                float v[BC];
                int q = 0;
#pragma unroll
                for (int c = 0; c < BC; ++c)
                    if ((rb >> c) & 1u) v[c] = a.bdata[k0 + q++];
                q = 0;
#pragma unroll
                for (int c = 0; c < BC; ++c)
                    if ((rb >> c) & 1u)
                        lst[pos0 + q++] = make_uint2(win_key(f0 + (uint32_t)c * fs, r), __float_as_uint(v[c]));
            }
        }
        lpos += ltot;
        gpos += gtot;
    }
    if (!ok || lpos + gpos + nrem > kWinList) return false;
    // remainder entries, row-sorted already: compacted into window / global
    for (int t0 = 0; t0 < nrem; t0 += 32) {
        const int q = t0 + lane;
        const bool valid = q < nrem;
        int32_t col;
        float val;
        if (t0 == 0) {
            col = rcol[0];
            val = rval[0];
        } else if (t0 == 32) {
            col = rcol[1];
            val = rval[1];
        } else {
            col = valid ? a.rem_col[j0 + q] : 0;
            val = valid ? a.rem_val[j0 + q] : 0.f;
        }
        const bool loc = valid && (uint32_t)(col - xb) < (uint32_t)kWinRows;
        const uint32_t mL = __ballot_sync(0xffffffffu, loc);
        const uint32_t mG = __ballot_sync(0xffffffffu, valid && !loc);
        const uint32_t below = (1u << lane) - 1u;
        if (valid) {
            const int32_t i = j0 + q;
            int r = 0;
#pragma unroll
            for (int r2 = 1; r2 < BR; ++r2) r += rstart[r2] <= i ? 1 : 0;
            if (loc) {
                lst[lpos + __popc(mL & below)] =
                    make_uint2(win_key((uint32_t)(col - xb) * 16u, r), __float_as_uint(val));
            } else {
                lst[kWinList - gpos - __popc(mG) + __popc(mG & below)] =
                    make_uint2(win_key((uint32_t)col * K4, r), __float_as_uint(val));
            }
        }
        lpos += __popc(mL);
        gpos += __popc(mG);
    }
    __syncwarp();
    // global entries first (deep gather batches), then the window's
    const int c4 = (lane & 15) * 4;
    float* ht = tile + h * BR * kWinCols + c4;   // this lane's 4 columns of its half-warp's tile
    win_walk<kWinGather>(lst + (kWinList - gpos), gpos, reinterpret_cast<const float4*>(Xg), ht, touched, h);
    win_walk<4>(lst, lpos, reinterpret_cast<const float4*>(xw + c4), ht, touched, h);
    __syncwarp();
    return true;
}

// Sum of the two half-warp tiles' row r for this lane's 4 columns (rows a
// half-warp did not touch count as zero).
template <int BR>
__device__ __forceinline__ float4 win_row(const float* tile, int r, int c4, uint32_t t0m, uint32_t t1m) {
    float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((t0m >> r) & 1u) y = *reinterpret_cast<const float4*>(tile + r * kWinCols + c4);
    if ((t1m >> r) & 1u) {
        const float4 z = *reinterpret_cast<const float4*>(tile + (BR + r) * kWinCols + c4);
        y.x += z.x;
        y.y += z.y;
        y.z += z.z;
        y.w += z.w;
    }
    return y;
}

// 96 registers: two CTAs of 288 threads per SM put five warps on one SM
// sub-partition, whose register file (16 K) then allows at most 102 per
// thread.
template <int BR>
__global__ void __maxnreg__(GL_WIN_MAXREG) window_kernel(const StripeArgs<float> a) {
    using SM = WinSmem<BR>;
    extern __shared__ __align__(128) unsigned char smem[];
    float* const xwin = reinterpret_cast<float*>(smem + SM::xwin);
    int32_t* const winfo = reinterpret_cast<int32_t*>(smem + SM::winfo);
    uint64_t* const full = reinterpret_cast<uint64_t*>(smem + SM::ctl);
    uint64_t* const empty = full + kWinBufs;
    int64_t* const unit_of = reinterpret_cast<int64_t*>(empty + kWinBufs);   // [bufs]
    int32_t* const xbase_of = reinterpret_cast<int32_t*>(unit_of + kWinBufs); // [bufs]
    int32_t* const take = xbase_of + kWinBufs;                                // [bufs] items handed out

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t BT = a.batch * a.ntiles;
    const int64_t npg = (a.num_pieces + kWinWarps - 1) / kWinWarps;   // piece groups
    const int64_t nwin = (a.rows + kWinRows - 1) / kWinRows;
    const int64_t units = (npg + nwin) * BT;
    constexpr int SPW = kWinRows / BR;                                 // stripes per window
    static_assert(SPW + 1 + SPW + kWinRows + 1 <= kWinInfo, "window info fits");
    int32_t* const err = reinterpret_cast<int32_t*>(a.sched + 2);

    if (threadIdx.x == 0) {
        for (int i = 0; i < kWinBufs; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], kWinWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == kWinWarps) {
        // ---- producer ---------------------------------------------------------
        for (int64_t k = 0;; ++k) {
            const int buf = (int)(k % kWinBufs);
            const int64_t use = k / kWinBufs;
            if (use >= 1 && !mbar_wait(&empty[buf], (uint32_t)((use - 1) & 1))) {
                if (lane == 0) atomicExch(err, GL_ERR_TIMEOUT);
                // let the copies already issued land before the CTA can exit
                // (bounded as well)
                for (int64_t kk = k - kWinBufs + 1; kk < k; ++kk)
                    if (kk >= 0) mbar_wait(&full[kk % kWinBufs], (uint32_t)((kk / kWinBufs) & 1));
                break;
            }
            unsigned long long u = 0;
            if (lane == 0) u = atomicAdd(a.sched, 1ull);
            u = __shfl_sync(0xffffffffu, u, 0);
            if ((int64_t)u >= units) {
                if (lane == 0) {
                    unit_of[buf] = -1;
                    mbar_arrive(&full[buf]);
                }
                break;
            }
            const int64_t bt = (int64_t)u % BT;
            const int64_t w = (int64_t)u / BT;
            const int64_t b = bt / a.ntiles;
            const int tile = (int)(bt - b * a.ntiles);
            int64_t xb;
            int32_t* info = winfo + buf * kWinInfo;
            if (w < npg) {
                const int32_t hh = a.piece_heavy[w * kWinWarps];
                xb = ((int64_t)a.heavy_stripe[hh] * BR) / kWinRows * kWinRows;
            } else {
                // the window's stripe pointers, heavy flags and row pointers,
                // so the consumers start their stripes from shared memory:
                // info[0..SPW] stripe_ptr, info[SPW+1..2SPW] heavy_of,
                // info[2SPW+1..2SPW+1+64] rem_ptr (clamped to the matrix)
                xb = (w - npg) * kWinRows;
                const int64_t s0 = xb / BR;
                for (int i = lane; GL_WIN_PREFETCH_INFO && i < kWinInfo; i += 32) {
                    int32_t v = 0;
                    if (i <= SPW) {
                        const int64_t s = s0 + i < a.nstripes ? s0 + i : a.nstripes;
                        v = a.stripe_ptr[s];
                    } else if (i <= 2 * SPW) {
                        const int64_t s = s0 + (i - SPW - 1);
                        v = (a.heavy_of != nullptr && s < a.nstripes) ? a.heavy_of[s] : -1;
                    } else if (i <= 2 * SPW + 1 + kWinRows) {
                        const int64_t r = xb + (i - 2 * SPW - 1);
                        v = a.rem_ptr[r < a.rows ? r : a.rows];
                    }
                    info[i] = v;
                }
            }
            const int64_t nx = a.cols - xb < kWinRows ? (a.cols - xb > 0 ? a.cols - xb : 0) : kWinRows;
            const int tw = (a.K - tile * kWinCols) < kWinCols ? (a.K - tile * kWinCols) : kWinCols;
            const uint32_t bytes = (uint32_t)(nx * tw * 4);
            float* dst = xwin + buf * (kWinRows * kWinCols);
            const float* src = a.X + (b * a.cols + xb) * (int64_t)a.K + tile * kWinCols;
            __syncwarp();
            if (lane == 0) {
                unit_of[buf] = (int64_t)u;
                xbase_of[buf] = (int32_t)xb;
                take[buf] = 0;
                mbar_arrive_expect_tx(&full[buf], bytes);
            }
            __syncwarp();
            if (bytes > 0) {
                if (a.K == kWinCols) {   // the window's rows are contiguous: one copy
                    if (lane == 0) bulk_load(dst, src, bytes, &full[buf]);
                } else {
                    for (int64_t r = lane; r < nx; r += 32)
                        bulk_load(dst + r * kWinCols, src + r * a.K, (uint32_t)(tw * 4), &full[buf]);
                }
            }
        }
        if (lane == 0) {
            // the last producer to finish resets the scheduler for the next launch
            __threadfence();
            if (atomicAdd(a.sched + 1, 1ull) == (unsigned long long)gridDim.x - 1) {
                a.sched[0] = 0;
                a.sched[1] = 0;
                __threadfence();
            }
        }
        return;
    }

    // ---- consumers ------------------------------------------------------------
    uint2* const lst = reinterpret_cast<uint2*>(smem + SM::lists) + (size_t)warp * kWinList;
    float* const tile = reinterpret_cast<float*>(smem + SM::tiles) + (size_t)warp * 2 * BR * kWinCols;
    int32_t* const rstart = reinterpret_cast<int32_t*>(smem + SM::rinfo) + warp * 16;
    const int h = lane >> 4;
    const int c4 = (lane & 15) * 4;

    for (int64_t k = 0;; ++k) {
        const int buf = (int)(k % kWinBufs);
        if (!mbar_wait(&full[buf], (uint32_t)((k / kWinBufs) & 1))) {
            if (lane == 0) atomicExch(err, GL_ERR_TIMEOUT);
            break;
        }
        const int64_t u64 = unit_of[buf];
        if (u64 < 0) break;
        // unit numbers, windows and batch x tile indices fit 32 bits (fewer
        // live registers across the list walks)
        const uint32_t u = (uint32_t)u64;
        const int32_t xb = xbase_of[buf];
        const float* xw = xwin + buf * (kWinRows * kWinCols);
        const int32_t* info = winfo + buf * kWinInfo;
        const uint32_t bt = u % (uint32_t)BT;
        const int64_t w = (int64_t)(u / (uint32_t)BT);
        const int32_t b = (int32_t)(bt / (uint32_t)a.ntiles);
        const int tile_i = (int)(bt - (uint32_t)b * (uint32_t)a.ntiles);
        const int col_base = tile_i * kWinCols + c4;
        const bool lane_ok = col_base < a.K;
        const float* Xg = a.X + (int64_t)b * a.cols * (int64_t)a.K + (lane_ok ? col_base : tile_i * kWinCols);
        const bool pieces = w < npg;
        const int items = pieces ? (int)((a.num_pieces - w * kWinWarps) < kWinWarps ? (a.num_pieces - w * kWinWarps)
                                                                                    : kWinWarps)
                                 : SPW;

        // items of the unit (stripes of the window, or pieces) are handed out
        // one at a time to whichever warp asks, so the warps stay balanced
        for (int it_static = warp;; it_static += kWinWarps) {
#if GL_WIN_DYNAMIC_ITEMS
            int it = 0;
            if (lane == 0) it = atomicAdd(&take[buf], 1);
            it = __shfl_sync(0xffffffffu, it, 0);
#else
            const int it = it_static;
#endif
            if (it >= items) break;
            // the item's ranges; rstart[0..BR] = first remainder entry of each
            // row, rstart[9] = first row, rstart[10] = rows, rstart[11] = piece
            // number or -1 (light stripe)
            int32_t b0, b1, j0, j1;
            if (pieces) {
                const int64_t p = w * kWinWarps + it;
                const int32_t hh = a.piece_heavy[p];
                const int64_t s = a.heavy_stripe[hh];
                const int64_t row0 = s * BR;
                const int nr = (int)(row0 + BR < a.rows ? BR : a.rows - row0);
                if (a.piece_range != nullptr) {
                    const int4 pr = *reinterpret_cast<const int4*>(a.piece_range + 4 * p);
                    b0 = pr.x;
                    b1 = pr.y;
                    j0 = pr.z;
                    j1 = pr.w;
                } else {
                    const int32_t pidx = (int32_t)(p - a.heavy_first[hh]);
                    const int32_t sb0 = a.stripe_ptr[s], sb1 = a.stripe_ptr[s + 1];
                    const int64_t pk0 = a.offsets[sb0];
                    const int64_t pw = (int64_t)a.offsets[sb1] - pk0;
                    const int32_t rj0 = a.rem_ptr[row0], rj1 = a.rem_ptr[row0 + nr];
                    const int64_t total = pw + (rj1 - rj0);
                    const int64_t u0 = (int64_t)pidx * a.piece_work;
                    const int64_t u1 = (u0 + a.piece_work < total) ? u0 + a.piece_work : total;
                    b0 = lower_bound_i32(a.offsets, sb0, sb1, pk0 + u0);
                    b1 = (u1 >= pw) ? sb1 : lower_bound_i32(a.offsets, sb0, sb1, pk0 + u1);
                    j0 = rj0 + (int32_t)(u0 > pw ? u0 - pw : 0);
                    j1 = rj0 + (int32_t)(u1 > pw ? u1 - pw : 0);
                }
                if (lane <= BR) {
                    int32_t rs = j1;
                    if (lane < nr) rs = a.rem_ptr[row0 + lane];
                    rs = rs < j0 ? j0 : (rs > j1 ? j1 : rs);
                    rstart[lane] = rs;
                }
                if (lane == 0) {
                    rstart[9] = (int32_t)row0;
                    rstart[10] = nr;
                    rstart[11] = (int32_t)p;
                }
            } else {
                const int64_t s = (w - npg) * SPW + it;
                if (s >= a.nstripes) continue;
                const int64_t row0 = s * BR;
                const int nr = (int)(row0 + BR < a.rows ? BR : a.rows - row0);
#if GL_WIN_PREFETCH_INFO
                if (info[SPW + 1 + it] >= 0) continue;   // heavy: done as pieces
                b0 = info[it];
                b1 = info[it + 1];
                const int32_t* rp = info + 2 * SPW + 1 + it * BR;   // rem_ptr of the stripe's rows
                j0 = rp[0];
                j1 = rp[nr];
                if (lane <= BR) rstart[lane] = lane <= nr ? rp[lane] : j1;
#else
                const int32_t hv = a.heavy_of != nullptr ? a.heavy_of[s] : -1;
                b0 = a.stripe_ptr[s];
                b1 = a.stripe_ptr[s + 1];
                int32_t rpl = 0;
                if (lane <= nr) rpl = a.rem_ptr[row0 + lane];
                if (hv >= 0) continue;
                j0 = __shfl_sync(0xffffffffu, rpl, 0);
                j1 = __shfl_sync(0xffffffffu, rpl, nr);
                if (lane <= BR) rstart[lane] = lane <= nr ? rpl : j1;
#endif
                if (lane == 0) {
                    rstart[9] = (int32_t)row0;
                    rstart[10] = nr;
                    rstart[11] = -1;
                }
            }
            __syncwarp();
            uint32_t touched = 0;
            if (!win_unit<BR>(a, b0, b1, j0, j1, rstart, xb, xw, Xg, lst, tile, touched, lane)) {
                if (lane == 0) atomicExch(err, GL_ERR_INVALID_ARGUMENT);
                continue;
            }
            const uint32_t t0m = __shfl_sync(0xffffffffu, touched, 0);
            const uint32_t t1m = __shfl_sync(0xffffffffu, touched, 16);
            const int64_t row0 = rstart[9];
            const int nr = rstart[10];
            const int64_t p = rstart[11];
            if (p < 0) {
                if (lane_ok) {
                    for (int r = h; r < nr; r += 2)
                        *reinterpret_cast<float4*>(a.Y + ((int64_t)b * a.rows + row0 + r) * (int64_t)a.K +
                                                   col_base) = win_row<BR>(tile, r, c4, t0m, t1m);
                }
            } else {
                // partial tile -> workspace; the last piece of the stripe reduces
                float* part = a.partial + (p * BT + bt) * BR * kWinCols;
                for (int r = h; r < BR; r += 2)
                    *reinterpret_cast<float4*>(part + r * kWinCols + c4) = win_row<BR>(tile, r, c4, t0m, t1m);
                __threadfence();
                __syncwarp();
                const int32_t hh = a.piece_heavy[p];
                const int32_t f0 = a.heavy_first[hh];
                const int32_t npieces = a.heavy_first[hh + 1] - f0;
                int last = 0;
                if (lane == 0) {
                    const int old = atomicAdd(a.counters + (int64_t)hh * BT + bt, 1);
                    last = (old == npieces - 1);
                    if (last) a.counters[(int64_t)hh * BT + bt] = 0;   // ready for the next call
                }
                last = __shfl_sync(0xffffffffu, last, 0);
                if (last) {
                    __threadfence();
                    for (int r = h; r < nr; r += 2) {
                        float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
                        for (int32_t q = 0; q < npieces; ++q) {
                            const float* pp =
                                a.partial + ((int64_t)(f0 + q) * BT + bt) * BR * kWinCols + r * kWinCols + c4;
                            const float4 z = __ldcg(reinterpret_cast<const float4*>(pp));
                            y.x += z.x;
                            y.y += z.y;
                            y.z += z.z;
                            y.w += z.w;
                        }
                        if (lane_ok)
                            *reinterpret_cast<float4*>(a.Y + ((int64_t)b * a.rows + row0 + r) * (int64_t)a.K +
                                                       col_base) = y;
                    }
                }
            }
            __syncwarp();
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[buf]);
    }
}

// Whether the window kernel serves this SpMM: FP32, whole float4 lanes
// (K % 4 == 0, 16-byte aligned X / Y), at least one full tile of columns, a
// workspace (the unit counter lives there), a load-balance schedule with
// pieces of at most kWinMaxPieceWork entries (so every item fits a warp's
// list), list keys (float4 index << 3) and unit numbers within 32 bits.
inline bool window_eligible(const StripeArgs<float>& a) {
    const uintptr_t xa = reinterpret_cast<uintptr_t>(a.X), ya = reinterpret_cast<uintptr_t>(a.Y);
    const int64_t units = (ceil_div(a.num_pieces, kWinWarps) + ceil_div(a.rows, kWinRows)) * a.batch *
                          ceil_div(a.K, kWinCols);
    return a.sched != nullptr && a.K >= kWinCols && a.K % 4 == 0 && xa % 16 == 0 && ya % 16 == 0 &&
           a.piece_work > 0 && a.piece_work <= kWinMaxPieceWork && a.rows < (int64_t(1) << 31) &&
           a.cols * (int64_t)(a.K / 4) < (int64_t(1) << 29) && units < (int64_t(1) << 31);
}

template <int BR>
int launch_window(const StripeArgs<float>& a0, cudaStream_t stream) {
    StripeArgs<float> a = a0;
    a.ntiles = (int32_t)ceil_div(a.K, kWinCols);
    const int64_t BT = a.batch * a.ntiles;
    const int64_t units = (ceil_div(a.num_pieces, kWinWarps) + ceil_div(a.rows, kWinRows)) * BT;
    if (units == 0) return GL_OK;
    auto kern = window_kernel<BR>;
    constexpr size_t smem = WinSmem<BR>::bytes;
    // shared-memory attribute and occupancy, once per device
    static std::atomic<int> occ_cache[kMaxDevices];
    int occ = 0;
    const int rc = per_device_value(
        occ_cache,
        [&](int* o) {
            GL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            // two CTAs of ~106 KB need the largest shared-memory carveout
            GL_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             (int)cudaSharedmemCarveoutMaxShared));
            GL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, kern, kWinThreads, smem));
            return GL_OK;
        },
        &occ);
    if (rc != GL_OK) return rc;
    int64_t blocks = (int64_t)num_sms() * occ;
    if (blocks > units) blocks = units;
    kern<<<(unsigned)blocks, kWinThreads, smem, stream>>>(a);
    GL_LAUNCH_CHECK("window_kernel");
    return GL_OK;
}

}  // namespace gl
