// Stripe-owning fused PBR-block + CSR-remainder kernel (sm_103a).
//
// Work unit: one warp owns one output stripe (block_rows consecutive rows)
// for one column tile.  The warp's 32 lanes form C column lanes x P nonzero
// lanes (C * P = 32): column lane c owns V consecutive columns of the tile
// (T = C * V columns per tile), and the P nonzero lanes split the stripe's
// entries between them.  The stripe's output tile [block_rows][T] lives in
// the warp's shared memory and is written to Y once — no atomics on the
// output, no pre-zeroed output, no second stream.
//
//   * decode: per chunk of 32 blocks the lanes take one block each
//     (metadata in registers, one packed warp scan of the per-row bit
//     counts) and write row-sorted (column, value) lists in shared memory,
//     followed by each row's CSR-remainder entries.  Values are packed in
//     row-major bit order, so a block's entries of one row are a contiguous
//     run.
//   * P <= 2 (32 or more columns): the warp walks one row at a time,
//     issuing GL_GATHER_DEPTH X-row gathers before their FMAs into one
//     V-wide accumulator, and adds the row to the tile.
//   * P > 2 (fewer than 32 columns, one column per lane): P consecutive
//     entries per round, one per group of C column lanes, summed per row by
//     a segmented warp scan.
//
// Load balance: stripes whose stored entries exceed 2 x piece_work (R-MAT
// hub rows reach tens of thousands) are cut into pieces of piece_work
// entries (packed values first, then remainder entries).  A piece is an
// independent work unit; each piece writes its partial tile to the caller's
// workspace, and the warp that finishes a stripe's last piece (detected with
// a per-stripe counter after a memory fence; nobody waits) adds the partials
// in piece order — so results are deterministic — and runs the epilogue.
//
// With PPR = true the epilogue is one power-iteration step instead of a
// plain store: X_out = alpha * (A X_in) + teleport terms, with the L1 change
// per column and the dangling mass of X_out accumulated in the same pass.
//
// The reference splits this work over two kernels on two streams with global
// atomics (kernels/pbr_kernel.cu:12-333 block kernels, :421-458 CSR kernel,
// bindings/bindings_kernels.cu:34-80 stream fork/join) and a separate update
// pass (kernels/ppr_kernel.cu:130-168).
#pragma once

#include "gl_common.cuh"

namespace gl {

constexpr int kStripeThreads = 256;
constexpr int kWinDrawRows = 64;   // rows per window of the window draw
constexpr int kWinDrawRing = 16;   // windows a CTA can have in flight

constexpr int kStripeWarps = kStripeThreads / 32;

// Workspace of one SpMM / power-iteration launch (caller-provided or the
// static scratch): [scheduler: 256 B][heavy-stripe counters][partial tiles].
// The first zero_bytes must be zero before the first launch; every launch
// leaves them zero again.
inline int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }
struct WorkspaceLayout {
    int64_t counters, partial, zero_bytes, total;
};
inline WorkspaceLayout workspace_layout(const gl_pbr_matrix* A, int64_t batch, int64_t K) {
    WorkspaceLayout w{};
    const bool heavy = A->num_pieces > 0;
    const int64_t elem = A->value_type == GL_F32 ? 4 : 8;
    const int64_t Kt = (K + 127) / 128 * 128;
    w.counters = 256;
    w.partial = w.counters + (heavy ? align256((int64_t)A->num_heavy * batch * K * 4) : 0);
    w.zero_bytes = w.partial;
    w.total = w.partial + (heavy ? align256((int64_t)A->num_pieces * batch * A->block_rows * Kt * elem) : 0);
    return w;
}

template <typename S, int V>
struct alignas(sizeof(S) * V) Pack {
    S v[V];
};

template <typename S>
struct StripeArgs {
    const int64_t* codes;
    const int32_t* coords;
    const int32_t* offsets;
    const S* bdata;
    const int32_t* rem_ptr;
    const int32_t* rem_col;
    const S* rem_val;
    const int32_t* stripe_ptr;
    int64_t rows, cols, nstripes, batch;
    int32_t K, ntiles;
    const S* X;
    S* Y;
    // heavy-stripe schedule (num_pieces == 0: every stripe is one unit)
    int32_t num_pieces, piece_work;
    const int32_t* heavy_of;       // [nstripes] heavy index or -1
    const int32_t* heavy_stripe;   // [num_heavy]
    const int32_t* heavy_first;    // [num_heavy + 1]
    const int32_t* piece_heavy;    // [num_pieces]
    const int32_t* piece_range;    // [num_pieces][4] block / remainder ranges, or nullptr
    S* partial;                    // [num_pieces][batch * ntiles][BR][T]
    int32_t* counters;             // [num_heavy][batch * ntiles], zero between calls
    // work distribution: units are drawn one at a time from sched[0];
    // sched[1] counts retired warps.  Both are zero between calls (the last
    // warp to retire resets them).  sched == nullptr: static round-robin
    // over the warps.
    unsigned long long* sched;
    // power-iteration epilogue
    const int32_t* tp_ptr;
    const int32_t* tp_row;
    const int32_t* tp_col;
    const float* tp_w;
    double alpha, tol;
    int32_t stop_mode, max_iter, step;
    const int32_t* chunk_base;
    double* res_hist;
    double* dang_hist;
    const uint32_t* dbitmap;
    int32_t dang_uniform;
    const double* col_alpha;       // [K] or nullptr: alpha for every column
    const double* col_tol;         // [K] or nullptr: tol for every column
    int32_t cta_sums;              // 1: per-column sums gathered per CTA in shared memory (2 * K doubles
                                   //    after the stripe buffers), one global atomic per CTA and column
    int32_t variant;               // gl_pbr_matrix.kernel: 0 automatic, 1 stripe kernel, 2 window kernel
    int32_t win_draw;              // 1: light stripes drawn window by window (needs sched)
};

template <typename S, int V>
__device__ __forceinline__ Pack<S, V> load_pack(const S* p) {
    return *reinterpret_cast<const Pack<S, V>*>(p);
}
template <typename S, int V>
__device__ __forceinline__ Pack<S, V> load_pack_cg(const S* p) {
    Pack<S, V> r;
#pragma unroll
    for (int j = 0; j < V; ++j) r.v[j] = __ldcg(p + j);
    return r;
}
template <typename S, int V>
__device__ __forceinline__ void store_pack(S* p, const Pack<S, V>& v) {
    *reinterpret_cast<Pack<S, V>*>(p) = v;
}

// Store of a finished output row (Y, or X_out of a power-iteration step):
// with GL_Y_EVICT_FIRST the row is marked first to leave L2 (it is not read
// again by this launch), keeping more of the gathered X rows resident.
#ifndef GL_Y_EVICT_FIRST
#define GL_Y_EVICT_FIRST 0
#endif
template <typename S, int V>
__device__ __forceinline__ void store_out(S* p, const Pack<S, V>& v) {
#if GL_Y_EVICT_FIRST
    if constexpr (sizeof(S) == 4 && V == 4) {
        unsigned long long pol;
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
        asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.v[0]),
                     "f"(v.v[1]), "f"(v.v[2]), "f"(v.v[3]), "l"(pol)
                     : "memory");
        return;
    } else if constexpr (sizeof(S) == 4 && V == 2) {
        unsigned long long pol;
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
        asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.v[0]), "f"(v.v[1]),
                     "l"(pol)
                     : "memory");
        return;
    }
#endif
    *reinterpret_cast<Pack<S, V>*>(p) = v;
}

// X-row gather: a plain load (GL_GATHER_LOAD 0), L2 only (1), or read-only
// without L1 allocation (2).  The L1 catches a fifth of the gathers and
// either bypass measured ~55 % slower, so 0 stays.
#ifndef GL_GATHER_LOAD
#define GL_GATHER_LOAD 0
#endif
// SpMM gathers (KEEP): the gathered X rows are marked to stay in L2 before
// other lines (evict_last).  The SpMM's X (268 MB at the 2^20 / 64-column
// shape) is reused row by row across stripes: 0.5634 -> 0.5572 ms.  The
// power-iteration step keeps plain loads: its iterate is many times the L2
// and the same hint made the 256-column step on 2^22 nodes 5 % slower.
#ifndef GL_SPMM_X_EVICT_LAST
#define GL_SPMM_X_EVICT_LAST 1
#endif
template <typename S, int V, bool KEEP = false>
__device__ __forceinline__ Pack<S, V> gather_pack(const S* p) {
    if constexpr (KEEP && GL_SPMM_X_EVICT_LAST && GL_GATHER_LOAD == 0 && sizeof(S) == 4 && (V == 4 || V == 2)) {
        unsigned long long pol;
        asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
        Pack<S, V> r;
        if constexpr (V == 4) {
            asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                         : "=f"(r.v[0]), "=f"(r.v[1]), "=f"(r.v[2]), "=f"(r.v[3]) : "l"(p), "l"(pol));
        } else {
            asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
                         : "=f"(r.v[0]), "=f"(r.v[1]) : "l"(p), "l"(pol));
        }
        return r;
    }
#if GL_GATHER_LOAD == 1
    Pack<S, V> r;
    if constexpr (sizeof(S) * V == 16) {
        const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
        static_assert(sizeof(r) == sizeof(v), "pack size");
        memcpy(&r, &v, sizeof(v));
    } else if constexpr (sizeof(S) * V == 8) {
        const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
        memcpy(&r, &v, sizeof(v));
    } else {
        r = load_pack_cg<S, V>(p);
    }
    return r;
#elif GL_GATHER_LOAD == 2
    Pack<S, V> r;
    if constexpr (sizeof(S) * V == 16) {
        float4 v;
        asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
                     : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p));
        memcpy(&r, &v, sizeof(v));
    } else {
        r = load_pack<S, V>(p);
    }
    return r;
#else
    return load_pack<S, V>(p);
#endif
}

// First index in [lo, hi) with offsets[idx] >= key (hi if none).
__device__ __forceinline__ int32_t lower_bound_i32(const int32_t* offsets, int32_t lo, int32_t hi, int64_t key) {
    while (lo < hi) {
        const int32_t mid = lo + ((hi - lo) >> 1);
        if ((int64_t)offsets[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// List machinery for P <= 2.  Decoding is lane-parallel (a few instructions
// per nonzero spread over the warp); consuming costs two broadcast shared
// loads, one address and V FMAs per nonzero, with the gathers of a batch all
// in flight before the first FMA.
// ---------------------------------------------------------------------------
#ifndef GL_LIST_CAP
#define GL_LIST_CAP 288
#endif
// entries per warp list (a chunk that does not fit goes row by row); small,
// because shared memory left unused goes to the L1 that catches repeated X
// rows (288 measured 2-7 % faster than 384, 512 slower)
constexpr int kListCap = GL_LIST_CAP;
// X-row gathers in flight per warp in the main batch (half that for 16-byte
// lanes); row tails go in batches of kTail
#ifndef GL_GATHER_DEPTH
#define GL_GATHER_DEPTH 16
#endif
constexpr int kTail = 4;
template <typename S, int V>
struct Gather {
    static constexpr int n = sizeof(S) * V >= 16 ? GL_GATHER_DEPTH / 2 : GL_GATHER_DEPTH;
};

// One list entry: column and value side by side, so one shared load brings
// both (two FP32 entries per 16-byte load).
template <typename S>
struct Entry;
template <>
struct alignas(8) Entry<float> {
    int32_t col;
    float val;
};
template <>
struct alignas(16) Entry<double> {
    int32_t col;
    int32_t pad;
    double val;
};
template <typename S>
__device__ __forceinline__ Entry<S> make_entry(int32_t col, S val) {
    Entry<S> e{};
    e.col = col;
    e.val = val;
    return e;
}
// During decode a block entry first holds the index of its value in
// block_data (so the value loads can be issued together afterwards).
__device__ __forceinline__ Entry<float> make_index_entry(int32_t col, int32_t k, float) {
    Entry<float> e;
    e.col = col;
    e.val = __int_as_float(k);
    return e;
}
__device__ __forceinline__ Entry<double> make_index_entry(int32_t col, int32_t k, double) {
    Entry<double> e;
    e.col = col;
    e.pad = k;
    e.val = 0.0;
    return e;
}
__device__ __forceinline__ int32_t entry_index(const Entry<float>& e) { return __float_as_int(e.val); }
__device__ __forceinline__ int32_t entry_index(const Entry<double>& e) { return e.pad; }

// NB gathers (entries e, e + P, ..., all issued before the first FMA) into
// the lane's V accumulators.  Lanes past the last column gather from a
// clamped (valid) address and never store.
template <typename S, int V, int P, int NB, bool KEEP>
__device__ __forceinline__ void gather_batch(S (&t)[V], const Entry<S>* lst, int e, const S* __restrict__ Xb,
                                             int32_t K) {
    Pack<S, V> x[NB];
    if constexpr (P == 1 && sizeof(S) == 4 && NB % 2 == 0) {
        // two entries per 16-byte broadcast load; the values are read again
        // after the gathers instead of holding NB more registers
        const int4* w = reinterpret_cast<const int4*>(lst + e);
#pragma unroll
        for (int q = 0; q < NB; q += 2) {
            const int4 c = w[q / 2];
            x[q] = gather_pack<S, V, KEEP>(Xb + (long long)c.x * K);
            x[q + 1] = gather_pack<S, V, KEEP>(Xb + (long long)c.z * K);
        }
#pragma unroll
        for (int q = 0; q < NB; q += 2) {
            const int4 c = w[q / 2];
#pragma unroll
            for (int j = 0; j < V; ++j) {
                t[j] = fma(__int_as_float(c.y), x[q].v[j], t[j]);
                t[j] = fma(__int_as_float(c.w), x[q + 1].v[j], t[j]);
            }
        }
    } else {
#pragma unroll
        for (int q = 0; q < NB; ++q) x[q] = gather_pack<S, V, KEEP>(Xb + (long long)lst[e + q * P].col * K);
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            const S v = lst[e + q * P].val;
#pragma unroll
            for (int j = 0; j < V; ++j) t[j] = fma(v, x[q].v[j], t[j]);
        }
    }
}

// Walks a list whose length is a multiple of kTail * P (padded with (0, 0)
// entries): main batches while they fill, then tail batches.  With P = 2 the
// two half-warps take alternate entries (each half-warp covers the whole
// column tile with V-wide loads).
template <typename S, int V, int P, bool KEEP>
__device__ __forceinline__ void consume_list(S (&t)[V], const Entry<S>* lst, int n_padded,
                                             const S* __restrict__ Xb, int32_t K, int p_lane) {
    constexpr int NG = Gather<S, V>::n;
    int e = p_lane;
    for (; e + (NG - 1) * P < n_padded; e += NG * P) gather_batch<S, V, P, NG, KEEP>(t, lst, e, Xb, K);
    for (; e < n_padded; e += kTail * P) gather_batch<S, V, P, kTail, KEEP>(t, lst, e, Xb, K);
}

// Pads the list [0, n) with (0, 0) entries up to a multiple of GR (never
// past kListCap, which is a multiple of it); returns the padded length.
template <typename S, int GR>
__device__ __forceinline__ int pad_list(Entry<S>* lst, int n, int lane) {
    const int np = (n + GR - 1) / GR * GR;
    if (lane < np - n) lst[n + lane] = make_entry<S>(0, S(0));
    __syncwarp();
    return np;
}

// Packed per-row counters: row r's count sits in 16-bit field r % 4 of word
// r / 4, so one 64-bit warp scan per word yields every row's offsets.
template <int BR>
struct RowPack {
    static constexpr int W = (BR + 3) / 4;
    uint64_t w[W];
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int i = 0; i < W; ++i) w[i] = 0;
    }
    __device__ __forceinline__ void set(int r, uint32_t v) { w[r >> 2] |= (uint64_t)v << (16 * (r & 3)); }
    __device__ __forceinline__ uint32_t get(int r) const { return (uint32_t)(w[r >> 2] >> (16 * (r & 3))) & 0xffffu; }
    // r not known at compile time: select the word without indexing registers
    __device__ __forceinline__ uint32_t get_dyn(int r) const {
        uint64_t x = w[0];
#pragma unroll
        for (int i = 1; i < W; ++i)
            if ((r >> 2) == i) x = w[i];
        return (uint32_t)(x >> (16 * (r & 3))) & 0xffffu;
    }
};

// Adds the lane's accumulators to row r of the tile (lane-owned columns)
// and clears them.
template <typename S, int V>
__device__ __forceinline__ void commit_row(S* tile_lane, int r, int T, S (&t)[V], bool own) {
    if (own) {
        Pack<S, V>* tp = reinterpret_cast<Pack<S, V>*>(tile_lane + r * T);
        Pack<S, V> o = *tp;
#pragma unroll
        for (int j = 0; j < V; ++j) o.v[j] += t[j];
        *tp = o;
    }
#pragma unroll
    for (int j = 0; j < V; ++j) t[j] = S(0);
}

// Walk for fewer than 32 columns (P = 32 / C > 2 entries per round, V = 1):
// in each round the P entry lanes take P consecutive list entries and their
// C column lanes gather one X element each; a segmented scan over the entry
// lanes (rows are sorted) sums each row's products, and the last lane of a
// row's segment adds the sum to the tile — deterministic, no atomics.
// Row of entry e: the number of rows r >= 1 starting at or before e
// (starts == nullptr: the whole list is row r_fixed).
template <typename S, int BR, int C>
__device__ __forceinline__ void consume_narrow(const Entry<S>* lst, int n, const int32_t* starts, int r_fixed,
                                               S* tile, int c_lane, int p_lane, bool own_col,
                                               const S* __restrict__ Xb, int32_t K) {
    constexpr int P = 32 / C;
    int32_t sv[BR];
#pragma unroll
    for (int r = 0; r < BR; ++r) sv[r] = starts != nullptr ? starts[r] : 0;
    for (int base = 0; base < n; base += 2 * P) {
        // two rounds per pass: both rounds' gathers in flight together
        S prod[2];
        int row[2];
        bool valid[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int e = base + h * P + p_lane;
            valid[h] = e < n;
            prod[h] = S(0);
            row[h] = r_fixed;
            if (valid[h]) {
                const Entry<S> en = lst[e];
                prod[h] = en.val * Xb[(long long)en.col * K];
                if (starts != nullptr) {
                    int r = 0;
#pragma unroll
                    for (int q = 1; q < BR; ++q) r += sv[q] <= e ? 1 : 0;
                    row[h] = r;
                }
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            S v = prod[h];
            const int r = row[h];
#pragma unroll
            for (int o = 1; o < P; o <<= 1) {
                const S u = __shfl_up_sync(0xffffffffu, v, o * C);
                const int ru = __shfl_up_sync(0xffffffffu, r, o * C);
                if (p_lane >= o && ru == r) v += u;
            }
            const int rn = __shfl_down_sync(0xffffffffu, r, C);
            const int e = base + h * P + p_lane;
            const bool last = valid[h] && (p_lane == P - 1 || e + 1 >= n || rn != r);
            if (last && own_col) tile[r * C + c_lane] += v;
            __syncwarp();
        }
    }
}

// Accumulation for P <= 2 into the warp's output tile in shared memory
// (tile[r * T + column], zeroed here, each lane its own columns).  Per chunk
// of 32 blocks: one packed warp scan of the per-row bit counts; if the
// chunk's rows (block entries + remainder entries) fit the list, every lane
// writes its block's entries for all rows at once, row-sorted, otherwise
// row by row (at most 32 x BC block entries per row, the remainder in
// list-sized pieces).  The rows are consumed one at a time (each padded to
// kTail * P entries) into a V-wide accumulator per lane; with P == 2 the two
// half-warps take alternate entries and are folded by one shuffle per row.
template <typename S, int BR, int BC, int V, int P, bool KEEP>
__device__ __forceinline__ void accumulate_rows(const StripeArgs<S>& a, S* tile, Entry<S>* lst, int32_t* rowinfo,
                                                int64_t s, int32_t b0, int32_t b1, int32_t j0, int32_t j1,
                                                const S* __restrict__ Xb, bool lane_ok, int lane, int p_lane,
                                                int c_lane, bool rp_known, int32_t rp) {
    constexpr uint32_t ROWMASK = (BC >= 32) ? 0xffffffffu : ((1u << BC) - 1u);
    constexpr bool NARROW = P > 2;
    constexpr int GR = NARROW ? 1 : kTail * P;   // row granule
    constexpr int T = (32 / P) * V;
    static_assert(kListCap % GR == 0 && kListCap >= 32 * BC + 2 * GR, "a row of one block chunk must fit the list");
    int32_t* rstart = rowinfo;
    int32_t* rlen = rowinfo + BR;
    int32_t* seg = rowinfo + 2 * BR;
    int32_t* blen = rowinfo + 3 * BR;
    const bool own = (p_lane == 0) && lane_ok;
    S* tile_lane = tile + c_lane * V;

    // remainder row ranges of this unit (lane r computes row r; rp_known:
    // lane r already holds rem_ptr of row r); zero the tile
    __syncwarp();
    const int32_t rp_next = __shfl_down_sync(0xffffffffu, rp, 1);
    if (lane < BR) {
        const int64_t row = s * BR + lane;
        int32_t rs = j1, re = j1;
        if (row < a.rows) {
            rs = rp_known ? rp : a.rem_ptr[row];
            re = rp_known ? rp_next : a.rem_ptr[row + 1];
            rs = rs > j0 ? rs : j0;
            re = re < j1 ? re : j1;
            re = re > rs ? re : rs;
        }
        rstart[lane] = rs;
        rlen[lane] = re - rs;
    }
    if (own) {
        Pack<S, V> z;
#pragma unroll
        for (int j = 0; j < V; ++j) z.v[j] = S(0);
#pragma unroll
        for (int r = 0; r < BR; ++r) store_pack<S, V>(tile_lane + r * T, z);
    }
    __syncwarp();

    for (int32_t kc = b0; kc < b1 || kc == b0; kc += 32) {
        const int32_t nb = (b1 - kc) < 32 ? (b1 - kc > 0 ? b1 - kc : 0) : 32;
        const bool last = kc + 32 >= b1;
        uint64_t code = 0;
        int32_t col0 = 0, off = 0;
        if (lane < nb) {
            code = static_cast<uint64_t>(a.codes[kc + lane]);
            col0 = a.coords[2 * (int64_t)(kc + lane) + 1];
            off = a.offsets[kc + lane];
        }
        if constexpr (P == 32) {
            // One column per tile: no list.  Lane b takes block kc + b whole
            // (its X values, then every stored value in row-major bit order
            // into one accumulator per block row), the chunk's remainder
            // entries are spread over the lanes, and a warp reduction per row
            // leaves the stripe's BR sums in lane 0, which adds them to the
            // tile (column 0 of each row).
            S acc[BR];
#pragma unroll
            for (int r = 0; r < BR; ++r) acc[r] = S(0);
            if (lane < nb) {
                S x[BC];
#pragma unroll
                for (int c = 0; c < BC; ++c)
                    x[c] = (int64_t)col0 + c < a.cols ? Xb[((int64_t)col0 + c) * a.K] : S(0);
                int32_t k = off;
#pragma unroll
                for (int r = 0; r < BR; ++r) {
#pragma unroll
                    for (int c = 0; c < BC; ++c) {
                        if ((code >> (r * BC + c)) & 1ull) {
                            acc[r] = fma(a.bdata[k], x[c], acc[r]);
                            ++k;
                        }
                    }
                }
            }
            if (last) {
                for (int32_t i = j0 + lane; i < j1; i += 32) {
                    int r = 0;
#pragma unroll
                    for (int r2 = 1; r2 < BR; ++r2) r += rstart[r2] <= i ? 1 : 0;
                    const S v = a.rem_val[i] * Xb[(int64_t)a.rem_col[i] * a.K];
#pragma unroll
                    for (int r2 = 0; r2 < BR; ++r2) acc[r2] += r2 == r ? v : S(0);
                }
            }
#pragma unroll
            for (int r = 0; r < BR; ++r) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
            }
            if (own) {
#pragma unroll
                for (int r = 0; r < BR; ++r) tile[r * T] += acc[r];
            }
            __syncwarp();
            if (kc >= b1) break;
            continue;
        }
        // per-row bit counts of this lane's block, scanned over the warp
        // (ex: entries of each row in earlier blocks of the chunk, packed)
        RowPack<BR> ex;
        ex.clear();
#pragma unroll
        for (int r = 0; r < BR; ++r) ex.set(r, __popc((uint32_t)(code >> (r * BC)) & ROWMASK));
        uint64_t tot_lane = 0;   // lane r / 4 holds the totals word r / 4 after this
#pragma unroll
        for (int i = 0; i < RowPack<BR>::W; ++i) {
            const uint64_t mine = ex.w[i];
            uint64_t v = mine;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            ex.w[i] = v - mine;
            const uint64_t t = __shfl_sync(0xffffffffu, v, 31);
            if ((lane >> 2) == i) tot_lane = t;
        }
        // row segments [block entries | remainder entries | row padding]:
        // lane r < BR owns row r; a scan over those lanes places them
        int32_t my_len = 0, my_blen = 0;
        if (lane < BR) {
            my_blen = (int32_t)((tot_lane >> (16 * (lane & 3))) & 0xffffu);
            my_len = my_blen + (last ? rlen[lane] : 0);
        }
        const int32_t padded = (my_len + GR - 1) / GR * GR;
        const int32_t incl_pad = (int32_t)warp_incl_scan_i64(padded);
        const int32_t total = __shfl_sync(0xffffffffu, incl_pad, BR - 1);
        if (lane < BR) {
            seg[lane] = incl_pad - padded;
            blen[lane] = my_blen;
        }
        __syncwarp();
        const bool fits = total <= kListCap;
        if (fits) {
            // Every entry is written once, complete (column, value), with
            // all lanes busy: the unit's remainder entries flat over
            // [j0, j1), the block entries as (block, row) pairs, one pair
            // per lane.  Loads of the first remainder rounds and of the
            // block values are issued before any of them is stored.
            const int32_t nrem = last ? j1 - j0 : 0;
            constexpr int kRemRounds = 2;
            int32_t rcol[kRemRounds];
            S rval[kRemRounds];
#pragma unroll
            for (int h = 0; h < kRemRounds; ++h) {
                const int q = h * 32 + lane;
                rcol[h] = q < nrem ? a.rem_col[j0 + q] : 0;
                rval[h] = q < nrem ? a.rem_val[j0 + q] : S(0);
            }
            const int npairs = nb * BR;
            for (int p0 = 0; p0 < npairs; p0 += 32) {
                const int p = p0 + lane;
                const int src = (p / BR) & 31;
                const int r = p % BR;
                const uint64_t bcode = __shfl_sync(0xffffffffu, code, src);
                const int32_t bcol0 = __shfl_sync(0xffffffffu, col0, src);
                const int32_t boff = __shfl_sync(0xffffffffu, off, src);
                uint64_t bex = 0;
#pragma unroll
                for (int i = 0; i < RowPack<BR>::W; ++i) {
                    const uint64_t w = __shfl_sync(0xffffffffu, ex.w[i], src);
                    if ((r >> 2) == i) bex = w;
                }
                const uint32_t rb = p < npairs ? (uint32_t)(bcode >> (r * BC)) & ROWMASK : 0u;
                if (rb) {
                    const int32_t k0 = boff + __popcll(bcode & ((1ull << (r * BC)) - 1ull));
                    const int32_t pos0 = seg[r] + (int32_t)((bex >> (16 * (r & 3))) & 0xffffu);
                    S v[BC];
                    int q = 0;
#pragma unroll
                    for (int c = 0; c < BC; ++c) {
                        if ((rb >> c) & 1u) {
                            v[c] = a.bdata[k0 + q];
                            ++q;
                        }
                    }
                    q = 0;
#pragma unroll
                    for (int c = 0; c < BC; ++c) {
                        if ((rb >> c) & 1u) {
                            lst[pos0 + q] = make_entry<S>(bcol0 + c, v[c]);
                            ++q;
                        }
                    }
                }
            }
            if (nrem > 0) {
                // row of remainder entry i: the rows r >= 1 starting at or
                // before it (row starts are non-decreasing)
                auto put = [&](int q, int32_t col, S val) {
                    const int32_t i = j0 + q;
                    int r = 0;
#pragma unroll
                    for (int r2 = 1; r2 < BR; ++r2) r += rstart[r2] <= i ? 1 : 0;
                    lst[seg[r] + blen[r] + (i - rstart[r])] = make_entry<S>(col, val);
                };
#pragma unroll
                for (int h = 0; h < kRemRounds; ++h)
                    if (h * 32 + lane < nrem) put(h * 32 + lane, rcol[h], rval[h]);
                for (int q = kRemRounds * 32 + lane; q < nrem; q += 32) put(q, a.rem_col[j0 + q], a.rem_val[j0 + q]);
            }
            if (GR > 1 && lane < BR) {   // row padding: lane r pads row r
                const int32_t len = blen[lane] + (last ? rlen[lane] : 0);
                const int32_t b = seg[lane];
                for (int32_t q = len; q < (len + GR - 1) / GR * GR; ++q) lst[b + q] = make_entry<S>(0, S(0));
            }
            __syncwarp();
            if constexpr (NARROW) {
                consume_narrow<S, BR, 32 / P>(lst, total, seg, 0, tile, c_lane, p_lane, lane_ok, Xb, a.K);
                __syncwarp();
                if (kc >= b1) break;
                continue;
            }
        }
#pragma unroll 1
        for (int r = 0; r < BR; ++r) {
            S t[V];
#pragma unroll
            for (int j = 0; j < V; ++j) t[j] = S(0);
            int base = 0, n;
            int32_t rs = 0, re = 0;   // remainder entries still to append (!fits)
            if (fits) {
                base = seg[r];
                n = (blen[r] + (last ? rlen[r] : 0) + GR - 1) / GR * GR;
            } else {
                uint32_t rb = (uint32_t)(code >> (r * BC)) & ROWMASK;
                if (rb) {
                    int pos = (int)ex.get_dyn(r);
                    int32_t k = off + (r == 0 ? 0 : __popcll(code & ((1ull << (r * BC)) - 1ull)));
                    while (rb) {
                        const int c = __ffs(rb) - 1;
                        rb &= rb - 1u;
                        lst[pos++] = make_index_entry(col0 + c, k++, S(0));
                    }
                }
                n = blen[r];
                __syncwarp();
                for (int q0 = 0; q0 < n; q0 += 128) {   // the row's block values
                    S v[4];
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        const int q = q0 + h * 32 + lane;
                        v[h] = q < n ? a.bdata[entry_index(lst[q])] : S(0);
                    }
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        const int q = q0 + h * 32 + lane;
                        if (q < n) lst[q].val = v[h];
                    }
                }
                if (last) {
                    rs = rstart[r];
                    re = rs + rlen[r];
                }
            }
            while (true) {
                if (!fits) {
                    __syncwarp();
                    const int room = kListCap - GR - n;
                    const int take = (re - rs) < room ? (re - rs) : room;
                    for (int q = lane; q < take; q += 32) lst[n + q] = make_entry<S>(a.rem_col[rs + q], a.rem_val[rs + q]);
                    n += take;
                    rs += take;
                    n = pad_list<S, GR>(lst, n, lane);
                }
                if constexpr (NARROW) {
                    consume_narrow<S, BR, 32 / P>(lst + base, n, nullptr, r, tile, c_lane, p_lane, lane_ok, Xb, a.K);
                } else {
                    consume_list<S, V, P, KEEP>(t, lst + base, n, Xb, a.K, p_lane);
                }
                if (rs >= re) break;
                __syncwarp();
                n = 0;
            }
            if constexpr (P == 2) {
#pragma unroll
                for (int j = 0; j < V; ++j) t[j] += __shfl_xor_sync(0xffffffffu, t[j], 16);
            }
            if constexpr (!NARROW) commit_row<S, V>(tile_lane, r, T, t, own);
            if (!fits) __syncwarp();   // the next row reuses the list
        }
        __syncwarp();
        if (kc >= b1) break;   // empty block range: one pass for the remainder
    }
}

// Dynamic shared memory of one CTA of stripe_kernel, per warp: the output
// tile [BR][T] (offset 0), the (column, value) list and the row bookkeeping.
template <typename S, int BR, int V, int C>
struct StripeSmem {
    static constexpr int P = 32 / C;
    static constexpr int T = C * V;
    static constexpr size_t tile = (size_t)kStripeWarps * BR * T * sizeof(S);
    static constexpr size_t list = (size_t)kStripeWarps * kListCap * sizeof(Entry<S>);
    static constexpr size_t info = (size_t)kStripeWarps * 4 * BR * sizeof(int32_t);
    static constexpr size_t bytes = tile + list + info;
    static_assert(tile % 16 == 0 && list % 16 == 0, "regions stay 16-byte aligned");
};

// Minimum resident CTAs per SM the register allocation must allow (64
// registers per thread at 4; the power-iteration epilogue with 16-byte lanes
// needs more).
#ifndef GL_STRIPE_MIN_CTAS
#define GL_STRIPE_MIN_CTAS 4
#endif
#ifndef GL_PPR_MIN_CTAS
#define GL_PPR_MIN_CTAS 3
#endif
// For at most 4 columns (one column per lane, up to 4 column lanes) 5 CTAs
// of 48 registers measured 7 % faster than 4 of 64, despite spills; wider
// narrow shapes lost.
#ifndef GL_NARROW_MIN_CTAS
#define GL_NARROW_MIN_CTAS 5
#endif
template <typename S, int V, bool PPR, int C>
struct MinBlocks {
    static constexpr int n = (PPR && sizeof(S) * V >= 16) ? GL_PPR_MIN_CTAS
                             : (C <= 4 ? GL_NARROW_MIN_CTAS : GL_STRIPE_MIN_CTAS);
};

// One column's terms of power-iteration step t: the alpha that scales A x,
// the teleport scale (1 - alpha, plus the dangling mass when it goes to the
// teleport vector), the uniform dangling share, and whether the column has
// converged (STOP_PER_COLUMN).
struct ColumnTerms {
    double alpha, scale, uniform;
    bool frozen;
};
template <typename S>
__device__ __forceinline__ ColumnTerms column_terms(const StripeArgs<S>& a, int t, int col) {
    ColumnTerms c;
    c.alpha = a.col_alpha != nullptr ? a.col_alpha[col] : a.alpha;
    const double tl = a.col_tol != nullptr ? a.col_tol[col] : a.tol;
    c.scale = 1.0 - c.alpha;
    c.uniform = 0.0;
    if (a.dbitmap != nullptr) {
        const double d = c.alpha * a.dang_hist[(int64_t)t * a.K + col];
        if (a.dang_uniform) c.uniform = d / (double)a.rows;
        else c.scale += d;
    }
    c.frozen = a.stop_mode == GL_PPR_STOP_PER_COLUMN && t > 0 && a.res_hist[(int64_t)(t - 1) * a.K + col] < tl;
    return c;
}

template <typename S, int BR, int BC, int V, int C, bool PPR>
__global__ void __launch_bounds__(kStripeThreads, MinBlocks<S, V, PPR, C>::n)
stripe_kernel(const StripeArgs<S> a) {
    constexpr int P = 32 / C;            // nonzero lanes per warp
    constexpr int T = C * V;             // columns per tile

    using SM = StripeSmem<S, BR, V, C>;
    extern __shared__ __align__(16) unsigned char xs_dyn[];
    __shared__ int s_skip;
    // window draw: stripes handed out to this CTA's warps, and the ring of
    // the CTA's drawn windows ((sequence << 32) | window)
    __shared__ unsigned int s_take;
    __shared__ unsigned long long s_ring[kWinDrawRing];
    const int warp = threadIdx.x >> 5;
    S* const otile = reinterpret_cast<S*>(xs_dyn) + (size_t)warp * BR * T;
    Entry<S>* const lst = reinterpret_cast<Entry<S>*>(xs_dyn + SM::tile) + (size_t)warp * kListCap;
    int32_t* const rowinfo = reinterpret_cast<int32_t*>(xs_dyn + SM::tile + SM::list) + (size_t)warp * 4 * BR;

    const int lane = threadIdx.x & 31;
    const int c_lane = lane % C;
    const int p_lane = lane / C;
    const int64_t warp_id = (int64_t)blockIdx.x * kStripeWarps + (threadIdx.x >> 5);
    const int64_t nwarps = (int64_t)gridDim.x * kStripeWarps;
    const int64_t BT = a.batch * a.ntiles;
    const int64_t units = (int64_t)a.num_pieces + a.nstripes;
    const int64_t items = units * BT;

    int t = 0;
    if constexpr (PPR) {
        t = *a.chunk_base + a.step;
        if (t >= a.max_iter) return;
        if (a.stop_mode == GL_PPR_STOP_ALL && t > 0) {
            if (threadIdx.x < 32) {
                double m = 0.0;
                const double* prev = a.res_hist + (int64_t)(t - 1) * a.K;
                for (int k = lane; k < a.K; k += 32) m = fmax(m, prev[k]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
                if (lane == 0) s_skip = (m < a.tol) ? 1 : 0;
            }
            __syncthreads();
            if (s_skip) return;
        }
        // STOP_PER_COLUMN: when every column stopped at step t - 1 or before
        // (residuals of steps t - 2 and t - 1 below its threshold), the step
        // that stopped it has already copied it into the other buffer, both
        // buffers hold every final value, and this launch has nothing to do.
        if (a.stop_mode == GL_PPR_STOP_PER_COLUMN && t >= 2) {
            if (threadIdx.x < 32) {
                bool all = true;
                const double* p1 = a.res_hist + (int64_t)(t - 1) * a.K;
                const double* p2 = a.res_hist + (int64_t)(t - 2) * a.K;
                for (int k = lane; k < a.K; k += 32) {
                    const double tl = a.col_tol ? a.col_tol[k] : a.tol;
                    all = all && p1[k] < tl && p2[k] < tl;
                }
                const bool skip = __all_sync(0xffffffffu, all);
                if (lane == 0) s_skip = skip ? 1 : 0;
            }
            __syncthreads();
            if (s_skip) return;
        }
    }

    // per-CTA column sums (residual, dangling) in shared memory behind the
    // stripe buffers: warps add their partials there, and the CTA adds one
    // value per column to the FP64 totals at the end
    double* const s_sums = reinterpret_cast<double*>(xs_dyn + SM::bytes);
    if constexpr (PPR) {
        if (a.cta_sums) {
            for (int i = threadIdx.x; i < 2 * a.K; i += kStripeThreads) s_sums[i] = 0.0;
            __syncthreads();
        }
    }

    int64_t cur_bt = -1;
    int cur_col = 0;
    bool cur_ok = false;
    float res_acc[V];
    float dang_acc[V];
#pragma unroll
    for (int j = 0; j < V; ++j) {
        res_acc[j] = 0.f;
        dang_acc[j] = 0.f;
    }

    auto flush = [&]() {
        if constexpr (PPR) {
            if (cur_bt >= 0 && cur_ok) {
#pragma unroll
                for (int j = 0; j < V; ++j) {
                    const int col = cur_col + j;
                    double* rdst = a.cta_sums ? s_sums + col : a.res_hist + (int64_t)t * a.K + col;
                    double* ddst = a.cta_sums ? s_sums + a.K + col : a.dang_hist + (int64_t)(t + 1) * a.K + col;
                    if (res_acc[j] != 0.f) atomicAdd(rdst, (double)res_acc[j]);
                    if (a.dbitmap != nullptr && dang_acc[j] != 0.f) atomicAdd(ddst, (double)dang_acc[j]);
                    res_acc[j] = 0.f;
                    dang_acc[j] = 0.f;
                }
            }
        }
    };

    // next work item: drawn from the counter, or static round-robin
    // Window draw: the heavy-stripe pieces are drawn one at a time from the
    // global counter (tile by tile); then the CTA works through 64-row
    // windows of light stripes (for one column tile each), its warps taking the
    // window's stripes in turn, so the X rows of the window's diagonal block
    // (most of its nonzeros on locality-ordered graphs) are gathered by
    // warps of one CTA close together in time and hit its L1.  The warp that
    // takes a window's first stripe draws the window from a second global
    // counter and publishes it in the ring; the others wait for it (bounded).
#ifndef GL_TILE_MAJOR_SPMM
#define GL_TILE_MAJOR_SPMM 0
#endif
    constexpr bool tile_major_items = PPR || GL_TILE_MAJOR_SPMM;
    constexpr int SPW = kWinDrawRows / BR;
    const int64_t nwin = (a.nstripes + SPW - 1) / SPW;
    bool phase_windows = false;
    if (a.win_draw) {
        if (threadIdx.x == 0) s_take = 0;
        if (threadIdx.x < kWinDrawRing) s_ring[threadIdx.x] = ~0ull;
        __syncthreads();
    }
    auto next_item = [&](int64_t cur) -> int64_t {
        if (a.sched == nullptr) return cur + nwarps;
        unsigned long long v = 0;
        if (!a.win_draw) {
            if (lane == 0) v = atomicAdd(a.sched, 1ull);
            return (int64_t)__shfl_sync(0xffffffffu, v, 0);
        }
        // item number of (unit, batch x tile) in this launch's numbering
        auto item_of = [&](int64_t unit, int64_t btile) -> unsigned long long {
            return (unsigned long long)(tile_major_items ? btile * units + unit : unit * BT + btile);
        };
        if (lane == 0) {
            v = items;   // done unless a unit is found
            if (!phase_windows) {
                const unsigned long long p = atomicAdd(a.sched, 1ull);
                if ((int64_t)p < (int64_t)a.num_pieces * BT) {
                    v = item_of((int64_t)p % a.num_pieces, (int64_t)p / a.num_pieces);   // pieces tile by tile
                } else {
                    phase_windows = true;
                }
            }
            while (phase_windows) {
                const unsigned int tk = atomicAdd(&s_take, 1u);
                const unsigned int wl = tk / SPW, j = tk % SPW;
                volatile unsigned long long* slot = &s_ring[wl % kWinDrawRing];
                unsigned long long w;
                if (j == 0) {
                    w = atomicAdd(a.sched + 3, 1ull);
                    *slot = ((unsigned long long)wl << 32) | (w & 0xffffffffull);
                } else {
                    const long long t0 = clock64();
                    unsigned long long e = *slot;
                    while ((e >> 32) != wl) {
                        if (clock64() - t0 > 4000000000LL) {   // about two seconds: record and stop
                            atomicExch(reinterpret_cast<int*>(a.sched + 2), GL_ERR_TIMEOUT);
                            e = ((unsigned long long)wl << 32) | 0xffffffffull;
                            break;
                        }
                        e = *slot;
                    }
                    w = e & 0xffffffffull;
                }
                if ((int64_t)w >= nwin * BT) break;                  // no windows left: done
                const int64_t st = ((int64_t)w % nwin) * SPW + j;     // windows tile by tile
                if (st < a.nstripes) {
                    v = item_of(a.num_pieces + st, (int64_t)w / nwin);
                    break;
                }
                // past the last stripe of the last window: take again
            }
        }
        return (int64_t)__shfl_sync(0xffffffffu, v, 0);
    };
    for (int64_t item = a.sched != nullptr ? next_item(0) : warp_id; item < items; item = next_item(item)) {
        // power-iteration steps number the items column-tile major, so a
        // warp's successive items mostly share a tile and its per-column
        // residual sums are flushed (atomically) a few times per launch, not
        // at nearly every item; the SpMM keeps a unit's tiles adjacent (the
        // second decode of a stripe finds its matrix data in L2)
        constexpr bool tile_major = tile_major_items;
        const int64_t u = tile_major ? item % units : item / BT;
        const int64_t bt = tile_major ? item / units : item - u * BT;
        const int64_t b = bt / a.ntiles;
        const int tile = (int)(bt - b * a.ntiles);
        const int col_base = tile * T + c_lane * V;
        const bool lane_ok = col_base < a.K;

        if constexpr (PPR) {
            // STOP_PER_COLUMN: a tile whose columns all stopped is not
            // recomputed.  Columns frozen at this step (residual of step t-1
            // below their threshold) are copied X_in -> X_out; once a column
            // was also frozen at the step before, both iterate buffers hold
            // its final values and the tile is skipped outright.
            if (a.stop_mode == GL_PPR_STOP_PER_COLUMN && t >= 1) {
                bool fz = true, st = true;
                if (lane_ok) {
#pragma unroll
                    for (int j = 0; j < V; ++j) {
                        const int col = col_base + j;
                        const double tl = a.col_tol != nullptr ? a.col_tol[col] : a.tol;
                        fz = fz && a.res_hist[(int64_t)(t - 1) * a.K + col] < tl;
                        st = st && t >= 2 && a.res_hist[(int64_t)(t - 2) * a.K + col] < tl;
                    }
                }
                const bool all_frozen = __all_sync(0xffffffffu, fz);
                if (all_frozen && __all_sync(0xffffffffu, st && fz)) continue;
                if (all_frozen) {
                    int64_t s_copy = -1;
                    if (u < a.num_pieces) {
                        const int32_t hc = a.piece_heavy[u];
                        if (u == a.heavy_first[hc]) s_copy = a.heavy_stripe[hc];   // the stripe's first piece copies
                    } else {
                        s_copy = u - a.num_pieces;
                        if (a.heavy_of != nullptr && a.heavy_of[s_copy] >= 0) s_copy = -1;   // done as pieces
                    }
                    if (s_copy >= 0 && lane_ok && p_lane == 0) {
                        for (int r = 0; r < BR; ++r) {
                            const int64_t row = s_copy * BR + r;
                            if (row < a.rows)
                                store_pack<S, V>(a.Y + row * a.K + col_base, load_pack<S, V>(a.X + row * a.K + col_base));
                        }
                    }
                    continue;
                }
            }
        }

        // ---- the unit: a light stripe or one piece of a heavy stripe -------
        int64_t s;
        int32_t b0, b1, j0, j1;
        int32_t h = -1, pidx = 0, npieces = 1;
        int32_t rp = 0;            // lane r <= BR: rem_ptr of the stripe's row r
        bool rp_known = false;
        if (u < a.num_pieces) {
            h = a.piece_heavy[u];
            s = a.heavy_stripe[h];
            const int32_t f0 = a.heavy_first[h];
            pidx = (int32_t)(u - f0);
            npieces = a.heavy_first[h + 1] - f0;
            const int32_t sb0 = a.stripe_ptr[s], sb1 = a.stripe_ptr[s + 1];
            const int64_t pk0 = a.offsets[sb0];
            const int64_t pw = (int64_t)a.offsets[sb1] - pk0;
            const int64_t last_row = (s * BR + BR < a.rows) ? s * BR + BR : a.rows;
            const int32_t rj0 = a.rem_ptr[s * BR], rj1 = a.rem_ptr[last_row];
            const int64_t total = pw + (rj1 - rj0);
            if (a.piece_range != nullptr) {
                const int4 pr = *reinterpret_cast<const int4*>(a.piece_range + 4 * u);
                b0 = pr.x;
                b1 = pr.y;
                j0 = pr.z;
                j1 = pr.w;
            } else {
                const int64_t u0 = (int64_t)pidx * a.piece_work;
                const int64_t u1 = (u0 + a.piece_work < total) ? u0 + a.piece_work : total;
                b0 = lower_bound_i32(a.offsets, sb0, sb1, pk0 + u0);
                b1 = (u1 >= pw) ? sb1 : lower_bound_i32(a.offsets, sb0, sb1, pk0 + u1);
                const int64_t r0 = u0 > pw ? u0 - pw : 0;
                const int64_t r1 = u1 > pw ? u1 - pw : 0;
                j0 = rj0 + (int32_t)r0;
                j1 = rj0 + (int32_t)r1;
            }
        } else {
            // every load of the stripe's setup issued before the first use
            // (one memory round trip): heavy flag, block range, and the
            // remainder row pointers, lane r holding row r's
            s = u - a.num_pieces;
            const int nr = (int)(s * BR + BR < a.rows ? BR : a.rows - s * BR);
            const int32_t hv = a.heavy_of != nullptr ? a.heavy_of[s] : -1;
            b0 = a.stripe_ptr[s];
            b1 = a.stripe_ptr[s + 1];
            if (lane <= nr) rp = a.rem_ptr[s * BR + lane];
            if (hv >= 0) continue;   // done as pieces
            j0 = __shfl_sync(0xffffffffu, rp, 0);
            j1 = __shfl_sync(0xffffffffu, rp, nr);
            rp_known = true;
        }

        if constexpr (PPR) {
            if (bt != cur_bt) {
                flush();
                cur_bt = bt;
                cur_col = col_base;
                cur_ok = lane_ok && p_lane == 0;
            }
        }

        // lanes past the last column read a valid address and never store
        const S* __restrict__ Xb = a.X + b * a.cols * (int64_t)a.K + (lane_ok ? col_base : 0);

        accumulate_rows<S, BR, BC, V, P, !PPR>(a, otile, lst, rowinfo, s, b0, b1, j0, j1, Xb, lane_ok, lane, p_lane,
                                         c_lane, rp_known, rp);
        // from here on lane (c_lane, p_lane == 0) owns columns [c_lane * V, +V)
        // of every tile row

        // ---- heavy stripe: publish the partial; the last piece reduces ------
        if (h >= 0) {
            S* part = a.partial + ((int64_t)u * BT + bt) * BR * T + c_lane * V;
            if (p_lane == 0 && lane_ok) {
#pragma unroll 2
                for (int r = 0; r < BR; ++r)
                    store_pack<S, V>(part + r * T, load_pack<S, V>(otile + r * T + c_lane * V));
            }
            __threadfence();
            __syncwarp();
            int last = 0;
            if (lane == 0) {
                const int old = atomicAdd(a.counters + (int64_t)h * BT + bt, 1);
                last = (old == npieces - 1);
                if (last) a.counters[(int64_t)h * BT + bt] = 0;   // ready for the next call
            }
            last = __shfl_sync(0xffffffffu, last, 0);
            if (!last) continue;
            __threadfence();
            const int64_t first = (int64_t)a.heavy_first[h];
            if (p_lane == 0 && lane_ok) {
#pragma unroll 1
                for (int r = 0; r < BR; ++r) {
                    Pack<S, V> o;
#pragma unroll
                    for (int j = 0; j < V; ++j) o.v[j] = S(0);
                    for (int32_t q = 0; q < npieces; ++q) {
                        const Pack<S, V> x =
                            load_pack_cg<S, V>(a.partial + ((first + q) * BT + bt) * BR * T + c_lane * V + r * T);
#pragma unroll
                        for (int j = 0; j < V; ++j) o.v[j] += x.v[j];
                    }
                    store_pack<S, V>(otile + r * T + c_lane * V, o);
                }
            }
        }

        if (lane_ok && p_lane == 0) {
            const S* trow = otile + c_lane * V;

            // ---- epilogue --------------------------------------------------------
            if constexpr (!PPR) {
                S* Yb = a.Y + (b * a.rows) * (int64_t)a.K + col_base;
#pragma unroll 2
                for (int r = 0; r < BR; ++r) {
                    const int64_t row = s * BR + r;
                    if (row < a.rows) store_out<S, V>(Yb + row * a.K, load_pack<S, V>(trow + r * T));
                }
            } else {
                // this step's per-column terms (computed here, not kept in
                // registers across the accumulation)
                S alph[V], unif[V];
                bool frozen[V];
#pragma unroll
                for (int j = 0; j < V; ++j) {
                    const ColumnTerms ct = column_terms(a, t, col_base + j);
                    alph[j] = static_cast<S>(ct.alpha);
                    unif[j] = static_cast<S>(ct.uniform);
                    frozen[j] = ct.frozen;
                }
                S* tw = otile + c_lane * V;
#pragma unroll 2
                for (int r = 0; r < BR; ++r) {
                    Pack<S, V> o = load_pack<S, V>(tw + r * T);
#pragma unroll
                    for (int j = 0; j < V; ++j) o.v[j] = fma(alph[j], o.v[j], unif[j]);
                    store_pack<S, V>(tw + r * T, o);
                }
                const int32_t e0 = a.tp_ptr[s], e1 = a.tp_ptr[s + 1];
                for (int32_t e = e0; e < e1; ++e) {
                    const int rr = a.tp_row[e] - (int)(s * BR);
                    const int cc = a.tp_col[e] - col_base;
                    if (cc >= 0 && cc < V) {
                        const S sc = static_cast<S>(column_terms(a, t, col_base + cc).scale);
                        tw[rr * T + cc] = fma(static_cast<S>(a.tp_w[e]), sc, tw[rr * T + cc]);
                    }
                }
                const S* Xin = a.X + col_base;
                S* Xout = a.Y + col_base;
#pragma unroll 2
                for (int r = 0; r < BR; ++r) {
                    const int64_t row = s * BR + r;
                    if (row < a.rows) {
                        const Pack<S, V> old = load_pack<S, V>(Xin + row * a.K);
                        const Pack<S, V> y = load_pack<S, V>(tw + r * T);
                        const bool dang = a.dbitmap != nullptr && ((a.dbitmap[row >> 5] >> (row & 31)) & 1u);
                        Pack<S, V> o;
#pragma unroll
                        for (int j = 0; j < V; ++j) {
                            const S nv = frozen[j] ? old.v[j] : y.v[j];
                            o.v[j] = nv;
                            res_acc[j] += (float)fabs(nv - old.v[j]);
                            if (dang) dang_acc[j] += (float)nv;
                        }
                        store_out<S, V>(Xout + row * a.K, o);
                    }
                }
            }
        }
    }
    flush();
    if constexpr (PPR) {
        if (a.cta_sums) {
            __syncthreads();
            for (int c = threadIdx.x; c < a.K; c += kStripeThreads) {
                const double r = s_sums[c], d = s_sums[a.K + c];
                if (r != 0.0) atomicAdd(a.res_hist + (int64_t)t * a.K + c, r);
                if (a.dbitmap != nullptr && d != 0.0) atomicAdd(a.dang_hist + (int64_t)(t + 1) * a.K + c, d);
            }
        }
    }
    if (a.sched != nullptr && lane == 0) {
        // this warp draws nothing more; the last one to retire resets the
        // scheduler for the next launch (nobody waits on anybody)
        __threadfence();
        if (atomicAdd(a.sched + 1, 1ull) == (unsigned long long)nwarps - 1) {
            a.sched[0] = 0;
            a.sched[1] = 0;
            a.sched[3] = 0;
            __threadfence();
        }
    }
}

// Host-side launcher for one (S, PPR) family; picks the block shape, the
// vector width V and the column-lane count C.  Returns a GL_* status.
template <typename S, bool PPR>
int launch_stripe(const StripeArgs<S>& a0, int block_rows, int block_cols, int tile_hint, int lane_split,
                  cudaStream_t stream);

// Columns per tile the launcher will use for K columns (for workspace sizing).
template <typename S>
int stripe_tile_width(int64_t K, int tile_hint, const void* X, const void* Y);

}  // namespace gl
