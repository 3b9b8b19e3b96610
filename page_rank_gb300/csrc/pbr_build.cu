// PBR builder on the device (sm_103a): CSR -> 64-bit block bitmasks, packed
// values and a CSR remainder, bit-identical to the reference builder
// csr_to_pbr<index_t, scalar_t> (Backend/graph_link/pbr_matrix/pbr_matrix.cpp:
// 340-477) for canonical CSR input.
//
// Work split: a group of lanes per stripe (block_rows consecutive rows; four
// 8-lane groups per warp for blocks up to 8 rows).  Lane r walks row r of the
// stripe; because each row is column-sorted, the group merges the rows by
// block column (the minimum of the lanes' head block columns), which yields
// the stripe's distinct blocks in block-column order together with their
// bitmask, the CSR position of their first nonzero, and per-row counts.
// Groups draw their stripes from a counter.  Long stripes (more than
// kBigCountEntries entries to count, more than kSmallStripeBlocks distinct
// blocks to order) go to 1024-thread CTAs instead, which sort (or, in shared
// memory, rank) instead of merging; the count pass lists them for those
// kernels, hub stripes first.
//
// Three device passes:
//   count  — per stripe: distinct / kept blocks, packed values; per row:
//            remainder entries; CSR validation (range, strictly increasing);
//            the block records of merged stripes and the sorted order of
//            long ones are left in the workspace for the fill;
//   (scans of those counts; an exclusive running max of distinct blocks)
//   fill   — per stripe: take the blocks' records, reproduce the reference's
//            emit order (below), write codes / coords / offsets, then merge
//            once more to move the values into block_data or the remainder.
//
// Emit order.  The reference emits a stripe's kept blocks in the iteration
// order of a std::unordered_map<index_t, ...> keyed by the block index
// (truncated to index_t), constructed with a bucket hint of
// sqrt(number of column blocks) and clear()ed — which keeps its bucket array —
// after every stripe (pbr_matrix.cpp:374-376, 389, 402, 425).  That order is a
// deterministic function of the keys' insertion order and the bucket count:
//   * the hash of an integer key is the key itself (sign-extended to size_t),
//     the bucket is hash % bucket_count;
//   * a node inserted into an empty bucket goes to the front of the node
//     list; one inserted into a non-empty bucket goes to the front of that
//     bucket's run.  So with insertion times tau, the list is ordered by
//     (first tau of the node's bucket, descending) then (tau, descending);
//   * a rehash happens just before the insertion that would take the element
//     count to (last bucket count + 1) and re-inserts the existing nodes in
//     their list order — i.e. it renumbers tau by list position;
//   * bucket counts only grow, and clear() keeps them, so the bucket count a
//     stripe starts with depends only on the most elements any earlier stripe
//     held.
// The sequence of bucket counts is read, on the host, from the same standard
// library container (filled with dummy keys), so no prime table is assumed.
// The same standard library must build this library and the reference.

#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "gl_common.cuh"
#include "gl_scan.cuh"

namespace gl {
namespace {

constexpr int kBuildThreads = 256;
constexpr int kBuildWarps = kBuildThreads / 32;
constexpr int kMaxChain = 64;
constexpr int64_t kInf = INT64_MAX;

enum BuildFlag { kFlagRange = 0, kFlagNoncanon = 1, kFlagIndptr = 2, kNumFlags = 4 };

// Work lists of the CTA kernels.  The count pass lists the stripes that go to
// build_count_big_kernel and to build_fill_big_kernel; each list fills from
// the front with its huge stripes (more than kHugeEntries entries: R-MAT hub
// rows) and from the back with the others, and the CTAs draw from it through
// a counter, so the huge stripes start first and no CTA is left holding a
// run of hub stripes that a static stride gave it.  The draw order does not
// change the output: every stripe writes to places fixed by the scans.
enum BuildWork {
    kWorkCountHead = 0, kWorkCountTail = 1, kWorkCountDraw = 2,
    kWorkFillHead = 3, kWorkFillTail = 4, kWorkFillDraw = 5, kWorkFillWarpDraw = 6, kWorkCountWarpDraw = 7,
    kNumWork = 8
};
constexpr int64_t kHugeEntries = 4096;
// Stripes with up to this many distinct blocks are ordered by one warp
// (build_fill_kernel, O(m^2 / 32) comparisons per lane), bigger ones by a
// CTA (build_fill_big_kernel, O(m) sorts and scans with a fixed cost of a few
// dozen block-wide barriers).
#ifndef GL_BUILD_SMALL_BLOCKS
#define GL_BUILD_SMALL_BLOCKS 64
#endif
constexpr int kSmallStripeBlocks = GL_BUILD_SMALL_BLOCKS;

// Workspace layout (every region 256-byte aligned).
struct BuildWs {
    int32_t* flags;         // kNumFlags
    int32_t* work;          // kNumWork: list heads / tails and draw counters
    int32_t* count_list;    // nstripes: stripes for build_count_big_kernel
    int32_t* fill_list;     // nstripes: stripes for build_fill_big_kernel
    int64_t* stripe_m;      // nstripes + 1 : distinct blocks   -> exclusive scan
    int64_t* stripe_kept;   // nstripes + 1 : kept blocks       -> exclusive scan
    int64_t* stripe_packed; // nstripes + 1 : kept values       -> exclusive scan
    int64_t* stripe_prefmax;// nstripes + 1 : exclusive running max of stripe_m
    int64_t* row_rem;       // rows + 1     : remainder entries -> exclusive scan
    int64_t* chain;         // 2 * kMaxChain: (count, buckets) pairs
    int64_t* scan_scratch;  // scan_scratch_elems(max(nstripes, rows) + 1)
    // per distinct block (upper bound: nnz), indexed by stripe_m scan
    uint64_t* rec_code;
    int64_t*  rec_bcol;
    int32_t*  rec_ins;      // first-nonzero position, then insertion rank
    int32_t*  rec_tau;
    uint32_t* rec_bkt;
    int32_t*  rec_g;        // bucket-run head tau, later: value offset in the stripe
                            // (rec_tau later holds the output slot, -1 = dropped)
    int32_t*  rec_pos;      // list position
    int32_t*  rec_pops;     // popcount of the block code
    // big stripes: sort / scan scratch (same indexing)
    int32_t*  rec_k0;
    int32_t*  rec_v0;
    int32_t*  rec_k1;
    int32_t*  rec_v1;
    // big stripes: per-entry sort / scan scratch, indexed by CSR position
    int32_t*  ent_a;
    int32_t*  ent_b;
    int32_t*  ent_c;
    int32_t*  ent_d;
    int64_t bytes;
};

inline int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

BuildWs layout_ws(void* base, int64_t rows, int64_t nnz, int32_t br) {
    BuildWs w{};
    const int64_t ns = ceil_div(rows, br);
    const int64_t scan_n = scan_scratch_elems((ns > rows ? ns : rows) + 1);
    char* p = static_cast<char*>(base);
    int64_t off = 0;
    auto take = [&](int64_t bytes) { char* q = p ? p + off : nullptr; off += align256(bytes); return q; };
    w.flags = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * kNumFlags));
    w.work = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * kNumWork));
    w.count_list = reinterpret_cast<int32_t*>(take(4 * (ns > 0 ? ns : 1)));
    w.fill_list = reinterpret_cast<int32_t*>(take(4 * (ns > 0 ? ns : 1)));
    w.stripe_m = reinterpret_cast<int64_t*>(take(8 * (ns + 1)));
    w.stripe_kept = reinterpret_cast<int64_t*>(take(8 * (ns + 1)));
    w.stripe_packed = reinterpret_cast<int64_t*>(take(8 * (ns + 1)));
    w.stripe_prefmax = reinterpret_cast<int64_t*>(take(8 * (ns + 1)));
    w.row_rem = reinterpret_cast<int64_t*>(take(8 * (rows + 1)));
    w.chain = reinterpret_cast<int64_t*>(take(8 * 2 * kMaxChain));
    w.scan_scratch = reinterpret_cast<int64_t*>(take(8 * scan_n));
    const int64_t nr = nnz > 0 ? nnz : 1;
    w.rec_code = reinterpret_cast<uint64_t*>(take(8 * nr));
    w.rec_bcol = reinterpret_cast<int64_t*>(take(8 * nr));
    w.rec_ins = reinterpret_cast<int32_t*>(take(4 * nr));
    w.rec_tau = reinterpret_cast<int32_t*>(take(4 * nr));
    w.rec_bkt = reinterpret_cast<uint32_t*>(take(4 * nr));
    w.rec_g = reinterpret_cast<int32_t*>(take(4 * nr));
    w.rec_pos = reinterpret_cast<int32_t*>(take(4 * nr));
    w.rec_pops = reinterpret_cast<int32_t*>(take(4 * nr));
    w.rec_k0 = reinterpret_cast<int32_t*>(take(4 * nr));
    w.rec_v0 = reinterpret_cast<int32_t*>(take(4 * nr));
    w.rec_k1 = reinterpret_cast<int32_t*>(take(4 * nr));
    w.rec_v1 = reinterpret_cast<int32_t*>(take(4 * nr));
    w.ent_a = reinterpret_cast<int32_t*>(take(4 * nr));
    w.ent_b = reinterpret_cast<int32_t*>(take(4 * nr));
    w.ent_c = reinterpret_cast<int32_t*>(take(4 * nr));
    w.ent_d = reinterpret_cast<int32_t*>(take(4 * nr));
    w.bytes = off;
    return w;
}

// ---------------------------------------------------------------------------
// Warp merge of the rows of one stripe.  Lanes 0..br-1 hold a cursor into
// their row.  step() advances to the next distinct block column and returns
// (for every lane) the block column, the lane's first position and count in
// that block, and the block's code / first position over the whole stripe.
// ---------------------------------------------------------------------------
// G: lanes per stripe (a power of two >= block_rows); a warp merges 32 / G
// stripes at once, each group of G lanes with its own reductions.
template <int G>
__device__ __forceinline__ unsigned group_mask() {
    return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
}

template <typename I, int G = 32>
struct StripeMerge {
    const I* indices;
    int64_t p, end;          // this lane's cursor into its row
    int64_t row_start;
    int64_t prev_col;
    int br, bc, lane;        // lane: this thread's row within the stripe
    unsigned gmask;
    bool check;
    int bad_range, bad_order, bad_indptr;

    // Cursors are clamped to [0, nnz] so a malformed indptr cannot cause an
    // out-of-bounds read; the count pass flags it and the build is rejected.
    __device__ void init(const I* indptr, const I* idx, int64_t s, int64_t rows, int64_t nnz, int br_, int bc_,
                         bool chk) {
        indices = idx;
        br = br_;
        bc = bc_;
        lane = threadIdx.x & (G - 1);
        gmask = group_mask<G>();
        check = chk;
        bad_range = 0;
        bad_order = 0;
        bad_indptr = 0;
        const int64_t row = s * br + lane;
        if (lane < br && row < rows) {
            const int64_t a = (int64_t)indptr[row];
            const int64_t b = (int64_t)indptr[row + 1];
            if (a < 0 || b < a || b > nnz) bad_indptr = 1;
            if (row == 0 && a != 0) bad_indptr = 1;
            if (row + 1 == rows && b != nnz) bad_indptr = 1;
            p = a < 0 ? 0 : (a > nnz ? nnz : a);
            end = b < p ? p : (b > nnz ? nnz : b);
        } else {
            p = 0;
            end = 0;
        }
        row_start = p;
        prev_col = -1;
    }

    // Returns false when the stripe is exhausted.  FIRST: also reduce the
    // block's first CSR position over the warp.
    template <bool FIRST = true>
    __device__ bool step(int64_t cols, int64_t& bcol, uint64_t& code, int64_t& first,
                         int& my_count, int64_t& my_first) {
        const int64_t head = (p < end) ? (int64_t)indices[p] / bc : kInf;
        const int64_t cur = group_min_i64(head, gmask);
        if (cur == kInf) return false;
        uint64_t bits = 0;
        int cnt = 0;
        int64_t f = kInf;
        if (head == cur) {
            f = p;
            while (p < end) {
                const int64_t col = (int64_t)indices[p];
                if (col / bc != cur) break;
                if (check) {
                    if (col < 0 || col >= cols) bad_range = 1;
                    if (col <= prev_col) bad_order = 1;
                }
                prev_col = col;
                const int64_t bit = (int64_t)lane * bc + col % bc;
                if (bit >= 0 && bit < 64) bits |= 1ull << bit;
                ++cnt;
                ++p;
            }
        }
        bcol = cur;
        code = group_or_u64(bits, gmask);
        first = FIRST ? group_min_i64(f, gmask) : f;
        my_count = cnt;
        my_first = f;
        return true;
    }
};

// Entries of stripe s according to indptr (clamped to [0, nnz]).
template <typename I>
__device__ __forceinline__ int64_t stripe_entries(const I* indptr, int64_t s, int64_t rows, int64_t nnz, int br) {
    const int64_t r0 = s * br;
    const int64_t r1 = r0 + br < rows ? r0 + br : rows;
    int64_t a = (int64_t)indptr[r0], b = (int64_t)indptr[r1];
    a = a < 0 ? 0 : (a > nnz ? nnz : a);
    b = b < a ? a : (b > nnz ? nnz : b);
    return b - a;
}

// Stripes with more entries than this are counted by a whole CTA
// (build_count_big_kernel) instead of one warp's serial merge, whose time
// grows with the stripe's distinct blocks (one merge step each).  256 was the
// fastest of 128 / 256 / 384 / 512 / 2048 on a 2^20-row R-MAT graph.
#ifndef GL_BUILD_BIG_COUNT_ENTRIES
#define GL_BUILD_BIG_COUNT_ENTRIES 256
#endif
constexpr int64_t kBigCountEntries = GL_BUILD_BIG_COUNT_ENTRIES;

// Stripes the CTA kernels handle with at most this many entries keep their
// per-entry and per-block scratch in dynamic shared memory instead of the
// global workspace (each of their ~100 dependent passes then waits on
// shared-memory latency, not L2).  0 keeps all scratch global.
#ifndef GL_BUILD_SMEM_ENTRIES
#define GL_BUILD_SMEM_ENTRIES 1024
#endif
constexpr int kSmemEntries = GL_BUILD_SMEM_ENTRIES;

// Resident 1024-thread CTAs per SM the two CTA kernels are compiled for (and
// launched with): the count kernel keeps 64 registers (at 32 it spills and
// was 6 % slower), the fill kernel runs two CTAs per SM on 1024-entry shared
// scratch (faster than one CTA on 1536 or 2048 entries).
#ifndef GL_BUILD_COUNT_BIG_CTAS
#define GL_BUILD_COUNT_BIG_CTAS 1
#endif
#ifndef GL_BUILD_FILL_BIG_CTAS
#define GL_BUILD_FILL_BIG_CTAS 2
#endif

// The CTA kernels' radix-sort and scan tiles load the next tile's elements
// before working on the current one (0: after).
#ifndef GL_BUILD_SORT_PREFETCH
#define GL_BUILD_SORT_PREFETCH 1
#endif

// Long stripes held in shared scratch are put in block-column order by
// binary searches in the other rows instead of four radix passes.
#ifndef GL_BUILD_SMEM_RANK
#define GL_BUILD_SMEM_RANK 1
#endif

// The fill pass takes the block-column order of stripes sorted in the
// workspace by the count pass (their entry indices and run indices) instead
// of sorting them again.
#ifndef GL_BUILD_REUSE_COUNT_SORT
#define GL_BUILD_REUSE_COUNT_SORT 1
#endif

// The warp count keeps the block records of the stripes it merges (code,
// block column, first position) in the per-entry scratch, and the warp fill
// copies them instead of merging the stripe's rows once more.
#ifndef GL_BUILD_REUSE_COUNT_RECORDS
#define GL_BUILD_REUSE_COUNT_RECORDS 1
#endif

// Unroll factor of the CTA kernels' element loops (2 and 4 spilled in the
// fill kernel's 32 registers and were 2-6 % slower than 1).
#ifndef GL_BUILD_UNROLL
#define GL_BUILD_UNROLL 1
#endif
constexpr int kUnroll = GL_BUILD_UNROLL;

// Hands a warp its stripes: GL_BUILD_WARP_DRAW consecutive stripes per draw
// from a counter, so warps that drew cheap stripes come back for more (one
// per draw was fastest; a static stride over the grid's warps, 0, left warps
// waiting on a neighbour's run of long stripes).
#ifndef GL_BUILD_WARP_DRAW
#define GL_BUILD_WARP_DRAW 1
#endif
template <int G = 32>
struct WarpDraw {
    int32_t* counter;
    int64_t ns, s, end;
    __device__ WarpDraw(int32_t* c, int64_t n) : counter(c), ns(n), s(-1), end(-1) {}
    __device__ bool next() {
#if GL_BUILD_WARP_DRAW > 0
        if (++s >= end) {
            const int lead = (threadIdx.x & 31) & ~(G - 1);
            int b = 0;
            if ((threadIdx.x & 31) == lead) b = atomicAdd(counter, GL_BUILD_WARP_DRAW);
            b = __shfl_sync(group_mask<G>(), b, lead);
            s = b;
            end = (int64_t)b + GL_BUILD_WARP_DRAW;
        }
#else
        constexpr int kGroups = 32 / G;
        const int64_t ng = (int64_t)gridDim.x * (blockDim.x >> 5) * kGroups;
        s = s < 0 ? ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * kGroups + ((threadIdx.x & 31) / G)
                  : s + ng;
#endif
        return s < ns;
    }
};

// Appends stripe s to a work list (head slot `slot`, tail slot `slot + 1`).
__device__ __forceinline__ void list_push(int32_t* list, int32_t* work, int slot, int64_t ns, int64_t s, bool huge) {
    if (huge) list[atomicAdd(&work[slot], 1)] = (int32_t)s;
    else list[ns - 1 - atomicAdd(&work[slot + 1], 1)] = (int32_t)s;
}

// Next stripe of a work list for the calling CTA (huge stripes first), or -1
// once the list is exhausted.  Called by every thread of the CTA.
__device__ __forceinline__ int64_t list_draw(const int32_t* list, int32_t* work, int slot, int64_t ns, int* s_item) {
    if (threadIdx.x == 0) {
        const int d = atomicAdd(&work[slot + 2], 1);
        const int h = work[slot], tl = work[slot + 1];
        *s_item = d < h ? list[d] : (d - h < tl ? list[ns - 1 - (d - h)] : -1);
    }
    __syncthreads();
    const int64_t s = *s_item;
    __syncthreads();
    return s;
}
// count: four int32 arrays per entry
constexpr int kCountSmemBytes = 16 * kSmemEntries;
// fill: four int32 arrays per entry; per block (at most one per entry) two
// 64-bit and ten int32 arrays
constexpr int kFillSmemBytes = 16 * kSmemEntries + 56 * kSmemEntries;

// ---------------------------------------------------------------------------
// count: per stripe distinct / kept blocks and kept values; per row remainder
// entries; validation flags.
// ---------------------------------------------------------------------------
// G lanes per stripe (block_rows <= G), 32 / G stripes per warp at a time.
// With `rec` (block columns fit int32), the stripe's block records (code,
// block column, first position relative to the stripe) are kept in the
// per-entry scratch at the stripe's CSR range, for build_fill_kernel.
template <typename I, int G>
__global__ void __launch_bounds__(kBuildThreads)
build_count_kernel(const I* indptr, const I* indices, int64_t rows, int64_t cols, int64_t nnz, int br, int bc,
                   int min_nnz, int64_t nstripes, BuildWs w, bool rec) {
    const int lane = threadIdx.x & (G - 1);
    const unsigned gmask = group_mask<G>();
    for (WarpDraw<G> d(&w.work[kWorkCountWarpDraw], nstripes); d.next();) {
        const int64_t s = d.s;
        const int64_t ent = stripe_entries(indptr, s, rows, nnz, br);
        if (ent > kBigCountEntries) {   // build_count_big_kernel
            if (lane == 0) list_push(w.count_list, w.work, kWorkCountHead, nstripes, s, ent > kHugeEntries);
            continue;
        }
        StripeMerge<I, G> mg;
        mg.init(indptr, indices, s, rows, nnz, br, bc, true);
        int64_t m = 0, kept = 0, packed = 0, rem = 0;
        int64_t bcol, first, my_first;
        uint64_t code;
        int my_count;
        int64_t last_bcol = -1;
        int64_t e0 = (int64_t)indptr[s * br];
        e0 = e0 < 0 ? 0 : (e0 > nnz ? nnz : e0);
        while (mg.template step<(GL_BUILD_REUSE_COUNT_RECORDS != 0)>(cols, bcol, code, first, my_count, my_first)) {
            // A negative or out-of-order column makes block columns repeat;
            // the count is still finite and the flags reject the build.
            if (bcol <= last_bcol) mg.bad_order = 1;
            last_bcol = bcol;
            if (GL_BUILD_REUSE_COUNT_RECORDS && rec && lane == 0 && m < ent) {   // (m < ent: inside the range)
                w.ent_a[e0 + m] = (int32_t)(uint32_t)code;
                w.ent_b[e0 + m] = (int32_t)(uint32_t)(code >> 32);
                w.ent_c[e0 + m] = (int32_t)bcol;
                w.ent_d[e0 + m] = (int32_t)(first - e0);
            }
            ++m;
            const int pop = __popcll(code);
            if (pop >= min_nnz) {
                ++kept;
                packed += pop;
            } else {
                rem += my_count;
            }
        }
        if (lane == 0) {
            w.stripe_m[s] = m;
            w.stripe_kept[s] = kept;
            w.stripe_packed[s] = packed;
            if (m > kSmallStripeBlocks) list_push(w.fill_list, w.work, kWorkFillHead, nstripes, s, ent > kHugeEntries);
        }
        const int64_t row = s * br + lane;
        if (lane < br && row < rows) w.row_rem[row] = rem;
        if (__any_sync(gmask, mg.bad_range) && lane == 0) atomicOr(&w.flags[kFlagRange], 1);
        if (__any_sync(gmask, mg.bad_order) && lane == 0) atomicOr(&w.flags[kFlagNoncanon], 1);
        if (__any_sync(gmask, mg.bad_indptr) && lane == 0) atomicOr(&w.flags[kFlagIndptr], 1);
    }
}

__device__ __forceinline__ uint32_t key_bucket(int64_t key_value, bool key32, uint64_t buckets) {
    // std::hash of an integer is the value converted to size_t.
    const int64_t k = key32 ? (int64_t)(int32_t)(uint32_t)(uint64_t)key_value : key_value;
    return (uint32_t)((uint64_t)k % buckets);
}

// A team is the set of threads that orders one stripe with order_stripe: a
// warp, for stripes with up to kSmallStripeBlocks distinct blocks (bigger
// ones go through order_stripe_big).
// A warp holds 32 / TEAM teams, each ordering its own stripe.
template <int TEAM>
struct Team {
    static __device__ __forceinline__ int rank() { return threadIdx.x & (TEAM - 1); }
    static __device__ __forceinline__ void sync() { __syncwarp(group_mask<TEAM>()); }
};

constexpr int kBigThreads = 1024;

// Orders the records with insertion rank < present as the standard library's
// node list would under `buckets` (see the file comment); writes list
// positions to pos.  O(m^2 / TEAM).
template <int TEAM>
__device__ void list_order(int64_t s, int64_t ncb, bool key32, uint64_t buckets, int m, int present,
                           const int64_t* bcol, const int32_t* ins, const int32_t* tau, uint32_t* bkt,
                           int32_t* g, int32_t* pos) {
    const int tr = Team<TEAM>::rank();
    for (int e = tr; e < m; e += TEAM)
        if (ins[e] < present) bkt[e] = key_bucket(s * ncb + bcol[e], key32, buckets);
    Team<TEAM>::sync();
    for (int e = tr; e < m; e += TEAM) {
        if (ins[e] >= present) continue;
        int32_t head = tau[e];
        const uint32_t be = bkt[e];
        for (int f = 0; f < m; ++f)
            if (ins[f] < present && bkt[f] == be && tau[f] < head) head = tau[f];
        g[e] = head;
    }
    Team<TEAM>::sync();
    for (int e = tr; e < m; e += TEAM) {
        if (ins[e] >= present) continue;
        const int32_t ge = g[e], te = tau[e];
        int r = 0;
        for (int f = 0; f < m; ++f) {
            if (ins[f] >= present) continue;
            const int32_t gf = g[f];
            r += (gf > ge || (gf == ge && tau[f] > te)) ? 1 : 0;
        }
        pos[e] = r;
    }
    Team<TEAM>::sync();
}

// Records the distinct blocks of stripe s in block-column order (a group of
// G lanes): code, block column and first CSR position relative to the
// stripe start.
template <typename I, int G>
__device__ void record_blocks(const I* indptr, const I* indices, int64_t s, int64_t rows, int64_t cols, int64_t nnz,
                              int br, int bc, uint64_t* code_r, int64_t* bcol_r, int32_t* first_r) {
    const int lane = threadIdx.x & (G - 1);
    StripeMerge<I, G> mg;
    mg.init(indptr, indices, s, rows, nnz, br, bc, false);
    int64_t bcol, first, my_first;
    uint64_t code;
    int my_count;
    int j = 0;
    const int64_t base = (int64_t)indptr[s * br];
    while (mg.step(cols, bcol, code, first, my_count, my_first)) {
        if (lane == 0) {
            code_r[j] = code;
            bcol_r[j] = bcol;
            first_r[j] = (int32_t)(first - base);
        }
        ++j;
    }
}

// Moves the stripe's values into block_data / the remainder (a group of G
// lanes): slot[j] >= 0 is the output slot of kept block j, doff[j] its value
// offset.
template <typename I, typename S, int G>
__device__ void move_values(const I* indptr, const I* indices, const S* values, int64_t s, int64_t rows,
                            int64_t cols, int64_t nnz, int br, int bc, const int32_t* slot, const int32_t* doff,
                            int64_t packed_base, const int64_t* row_rem, S* out_data, I* out_rem_col,
                            S* out_rem_val) {
    const int lane = threadIdx.x & (G - 1);
    const unsigned gmask = group_mask<G>();
    StripeMerge<I, G> mg;
    mg.init(indptr, indices, s, rows, nnz, br, bc, false);
    const int64_t row = s * br + lane;
    int64_t rem_cursor = (lane < br && row < rows) ? row_rem[row] : 0;
    int64_t bcol, first, my_first;
    uint64_t code;
    int my_count;
    int j = 0;
    while (mg.template step<false>(cols, bcol, code, first, my_count, my_first)) {
        if (slot[j] >= 0) {
            int incl = my_count;   // inclusive scan over the group's rows
#pragma unroll
            for (int o = 1; o < G; o <<= 1) {
                const int u = __shfl_up_sync(gmask, incl, o, G);
                if (lane >= o) incl += u;
            }
            const int before = incl - my_count;
            const int64_t dst = packed_base + doff[j] + before;
            for (int i = 0; i < my_count; ++i) out_data[dst + i] = values[my_first + i];
        } else {
            for (int i = 0; i < my_count; ++i) {
                out_rem_col[rem_cursor + i] = indices[my_first + i];
                out_rem_val[rem_cursor + i] = values[my_first + i];
            }
            rem_cursor += my_count;
        }
        ++j;
    }
}

// ---------------------------------------------------------------------------
// Big stripes (more than kSmallStripeBlocks distinct blocks; R-MAT hub rows
// reach 17 k blocks in one stripe of the 2^20 graph): the same emit order,
// computed by one 1024-thread CTA in O(m) passes over global scratch instead
// of the warp path's O(m^2) comparisons:
//   * insertion ranks: a stable radix sort of the first CSR positions;
//   * per rehash phase: the participating records in insertion-rank order
//     (a scatter: the ranks are a permutation), a stable radix sort of that
//     sequence by bucket (so each bucket's run is in rank order), run starts
//     and lengths by scans, and the list position of each record as
//     (records in runs whose head ranks later) + (later records of its run);
//   * output slots and value offsets: exclusive scans of the kept flags and
//     popcounts in list order.
// ---------------------------------------------------------------------------
struct BigShared {
    int32_t rowstart[33];                  // stripe-local row starts (block_rows + 1)
    int32_t nruns;
    int32_t hist[256];                     // digit bases of the pass
    int32_t tile_tot[256];                 // digit counts of the tile
    int32_t wcnt[kBigThreads / 32][256];   // per-warp digit counts, then prefixes
    int32_t warp_tot[kBigThreads / 32];
    int32_t carry;
};

struct BigRecs {
    const uint64_t* code;
    const int64_t* bcol;
    int32_t* ins;
    int32_t* tau;
    uint32_t* bkt;
    int32_t* g;
    int32_t* pos;
    int32_t* pops;
    int32_t* k0;
    int32_t* v0;
    int32_t* k1;
    int32_t* v1;
};

// In-place block-wide scan of a[0, n) (1024 threads, tiles of 1024): an
// exclusive or inclusive sum, or (MAX) an inclusive max.
template <bool MAX>
__device__ void big_scan(BigShared& sh, int32_t* a, int n, bool inclusive) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int32_t ident = MAX ? INT32_MIN : 0;
    auto op = [](int32_t x, int32_t y) { return MAX ? (x > y ? x : y) : x + y; };
    if (t == 0) sh.carry = ident;
    __syncthreads();
    // Each tile's element is loaded one tile ahead (a[] may be global
    // scratch; the scan writes only the current tile).
    int32_t x_next = t < n ? a[t] : ident;
    for (int base = 0; base < n; base += kBigThreads) {
        const int i = base + t;
        const int32_t x = x_next;
        if (GL_BUILD_SORT_PREFETCH) x_next = i + kBigThreads < n ? a[i + kBigThreads] : ident;
        int32_t v = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v = op(u, v);
        }
        if (lane == 31) sh.warp_tot[warp] = v;
        __syncthreads();
        if (warp == 0) {
            int32_t wv = sh.warp_tot[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t u = __shfl_up_sync(0xffffffffu, wv, o);
                if (lane >= o) wv = op(u, wv);
            }
            sh.warp_tot[lane] = wv;   // inclusive over the warps
        }
        __syncthreads();
        const int32_t c = sh.carry;
        const int32_t incl = op(c, warp > 0 ? op(sh.warp_tot[warp - 1], v) : v);
        if (i < n) a[i] = (inclusive || MAX) ? incl : incl - x;
        if (!GL_BUILD_SORT_PREFETCH) x_next = i + kBigThreads < n ? a[i + kBigThreads] : ident;
        __syncthreads();
        if (t == 0) sh.carry = op(c, sh.warp_tot[kBigThreads / 32 - 1]);
        __syncthreads();
    }
}

// Stable LSD radix sort (8-bit digits) of (key, val) pairs, n elements, keys
// read as unsigned and below 2^bits.  Ping-pongs between (k, v) and (kt, vt)
// for an even number of passes, so the result ends in (k, v).
__device__ void big_sort(BigShared& sh, int32_t* k, int32_t* v, int32_t* kt, int32_t* vt, int n, int bits) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int passes = (bits + 7) / 8;
    if (passes < 2) passes = 2;
    if (passes & 1) ++passes;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = 8 * pass;
        const int32_t* ks = (pass & 1) ? kt : k;
        const int32_t* vs = (pass & 1) ? vt : v;
        int32_t* kd = (pass & 1) ? k : kt;
        int32_t* vd = (pass & 1) ? v : vt;
        if (t < 256) sh.hist[t] = 0;
        __syncthreads();
        {   // four keys in flight per thread (ks may be global scratch)
            int i = t;
            for (; i + 3 * kBigThreads < n; i += 4 * kBigThreads) {
                const uint32_t a0 = (uint32_t)ks[i], a1 = (uint32_t)ks[i + kBigThreads];
                const uint32_t a2 = (uint32_t)ks[i + 2 * kBigThreads], a3 = (uint32_t)ks[i + 3 * kBigThreads];
                atomicAdd(&sh.hist[(a0 >> shift) & 255u], 1);
                atomicAdd(&sh.hist[(a1 >> shift) & 255u], 1);
                atomicAdd(&sh.hist[(a2 >> shift) & 255u], 1);
                atomicAdd(&sh.hist[(a3 >> shift) & 255u], 1);
            }
            for (; i < n; i += kBigThreads) atomicAdd(&sh.hist[((uint32_t)ks[i] >> shift) & 255u], 1);
        }
        __syncthreads();
        if (warp == 0) {   // exclusive scan of the histogram: digit bases
            int32_t run = 0;
            for (int d0 = 0; d0 < 256; d0 += 32) {
                const int32_t x = sh.hist[d0 + lane];
                int32_t incl = x;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int32_t u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += u;
                }
                sh.hist[d0 + lane] = run + incl - x;
                run += __shfl_sync(0xffffffffu, incl, 31);
            }
        }
        __syncthreads();
        // the next tile's pair is loaded while this one is ranked (sources
        // and destinations are different arrays)
        int32_t key_next = 0, val_next = 0;
        if (GL_BUILD_SORT_PREFETCH && t < n) {
            key_next = ks[t];
            val_next = vs[t];
        }
        for (int base = 0; base < n; base += kBigThreads) {   // tiles in order: stable
            const int i = base + t;
            const bool ok = i < n;
            int32_t key, val;
            if (GL_BUILD_SORT_PREFETCH) {
                key = key_next;
                val = val_next;
                key_next = i + kBigThreads < n ? ks[i + kBigThreads] : 0;
                val_next = i + kBigThreads < n ? vs[i + kBigThreads] : 0;
            } else {
                key = ok ? ks[i] : 0;
                val = ok ? vs[i] : 0;
            }
            const int d = ok ? (int)(((uint32_t)key >> shift) & 255u) : 256;
            for (int q = lane; q < 256; q += 32) sh.wcnt[warp][q] = 0;
            __syncwarp();
            const unsigned peers = __match_any_sync(0xffffffffu, d);
            const int lrank = __popc(peers & ((1u << lane) - 1u));
            if (ok && lrank == 0) sh.wcnt[warp][d] = __popc(peers);
            __syncthreads();
            if (t < 256) {   // per digit: exclusive prefix over the warps
                int32_t run = 0;
                for (int w2 = 0; w2 < kBigThreads / 32; ++w2) {
                    const int32_t c = sh.wcnt[w2][t];
                    sh.wcnt[w2][t] = run;
                    run += c;
                }
                sh.tile_tot[t] = run;
            }
            __syncthreads();
            if (ok) {
                const int dst = sh.hist[d] + sh.wcnt[warp][d] + lrank;
                kd[dst] = key;
                vd[dst] = val;
            }
            __syncthreads();
            if (t < 256) sh.hist[t] += sh.tile_tot[t];
            __syncthreads();
        }
    }
}

// list_order for a big stripe: list positions (pos) of the records with
// insertion rank < present under `buckets`, given their ranks tau (a
// permutation of [0, present) over those records).
__device__ void list_order_big(BigShared& sh, int64_t s, int64_t ncb, bool key32, uint64_t buckets, int m,
                               int present, const BigRecs& r) {
    const int t = threadIdx.x;
    // The record arrays are distinct, and below they are reached only through
    // these pointers (and pointers passed on from them); saying so lets the
    // compiler keep several iterations' loads in flight (huge stripes keep
    // them in global memory, where each round trip costs hundreds of cycles).
    const int64_t* __restrict__ bcol = r.bcol;
    const int32_t* __restrict__ ins = r.ins;
    const int32_t* __restrict__ tau = r.tau;
    uint32_t* __restrict__ bkt = r.bkt;
    int32_t* __restrict__ g = r.g;
    int32_t* __restrict__ pos = r.pos;
    int32_t* __restrict__ k0 = r.k0;
    int32_t* __restrict__ v0 = r.v0;
    int32_t* __restrict__ k1 = r.k1;
    int32_t* __restrict__ v1 = r.v1;
#pragma unroll kUnroll
    for (int e = t; e < m; e += kBigThreads) {
        if (ins[e] >= present) continue;
        const uint32_t b = key_bucket(s * ncb + bcol[e], key32, buckets);
        bkt[e] = b;
        v0[tau[e]] = e;   // records in rank order
    }
    __syncthreads();
#pragma unroll kUnroll
    for (int i = t; i < present; i += kBigThreads) k0[i] = (int32_t)bkt[v0[i]];
    __syncthreads();
    const int bits = buckets > 1 ? 64 - __clzll((long long)(buckets - 1)) : 1;
    big_sort(sh, k0, v0, k1, v1, present, bits);   // bucket runs, each in rank order
#pragma unroll kUnroll
    for (int i = t; i < present; i += kBigThreads) k1[i] = (i == 0 || k0[i] != k0[i - 1]) ? i : -1;
    __syncthreads();
    big_scan<true>(sh, k1, present, true);   // k1[i] = first sorted index of i's run
#pragma unroll kUnroll
    for (int i = t; i < present; i += kBigThreads) {
        const bool last = (i + 1 == present) || (k0[i + 1] != k0[i]);
        if (last) v1[k1[i]] = i - k1[i] + 1;   // run length, at the run start
    }
    __syncthreads();
    // head rank of each record's run, and its later run-mates
#pragma unroll kUnroll
    for (int i = t; i < present; i += kBigThreads) {
        const int e = v0[i];
        const int st = k1[i];
        g[e] = tau[v0[st]];
        pos[e] = v1[st] - 1 - (i - st);
    }
    __syncthreads();
    // run sizes indexed by head rank, inclusive prefix: records in runs whose
    // head is at most h; the runs with later heads come first in the list
#pragma unroll kUnroll
    for (int h = t; h < present; h += kBigThreads) k0[h] = 0;
    __syncthreads();
#pragma unroll kUnroll
    for (int i = t; i < present; i += kBigThreads)
        if (k1[i] == i) k0[tau[v0[i]]] = v1[i];
    __syncthreads();
    big_scan<false>(sh, k0, present, true);
    const int32_t total = present;
#pragma unroll kUnroll
    for (int e = t; e < m; e += kBigThreads)
        if (ins[e] < present) pos[e] += total - k0[g[e]];
    __syncthreads();
}

// Stripe-local row of entry i (rowstart[0..br] in shared memory).
__device__ __forceinline__ int big_row_of(const BigShared& sh, int br, int i) {
    int lo = 0, hi = br;   // rowstart[lo] <= i < rowstart[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (sh.rowstart[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The stripe's entries, stable-sorted by block column: sorted keys in a,
// stripe-local entry indices (CSR order) in b; c / d are scratch.
struct BigEntries {
    int32_t* a;
    int32_t* b;
    int32_t* c;
    int32_t* d;
};

// Stable block-column order of a stripe whose scratch is in shared memory
// (n <= kSmemEntries), without the radix passes: the block columns go to c in
// CSR order, then entry j of row r with block column k has j + (entries of
// earlier rows with block column <= k) + (entries of later rows with block
// column < k) entries before it — one binary search per other row in shared
// memory.  Leaves the block columns in rank order in a and the stripe-local
// entry indices in b, as the sort does.  b is first filled with the identity
// and ranks are clamped to [0, n), so rows that are not sorted (input the
// count pass then rejects) leave every index in range.  Columns are clamped
// to [0, cols); sh.rowstart holds the row starts.
template <typename I>
__device__ void big_rank_smem(const BigShared& sh, const I* indices, int64_t e0, int n, int br, int bc,
                              int64_t cols, const BigEntries& en) {
    const int t = threadIdx.x;
    for (int i = t; i < n; i += kBigThreads) {
        int64_t col = (int64_t)indices[e0 + i];
        col = col < 0 ? 0 : (col >= cols ? cols - 1 : col);
        en.c[i] = (int32_t)(col / bc);
        en.a[i] = 0;
        en.b[i] = i;
    }
    __syncthreads();
    int32_t key[kSmemEntries / kBigThreads + 1];
    int rank[kSmemEntries / kBigThreads + 1];
#pragma unroll
    for (int u = 0; u * kBigThreads < kSmemEntries; ++u) {
        const int i = t + u * kBigThreads;
        if (i >= n) break;
        const int r = big_row_of(sh, br, i);
        const int32_t k = en.c[i];
        int rk = i - sh.rowstart[r];
        for (int q = 0; q < br; ++q) {
            if (q == r) continue;
            const int q0 = sh.rowstart[q];
            int lo = q0, hi = sh.rowstart[q + 1];
            if (q < r) {   // entries with block column <= k
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (en.c[mid] <= k) lo = mid + 1;
                    else hi = mid;
                }
            } else {       // entries with block column < k
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (en.c[mid] < k) lo = mid + 1;
                    else hi = mid;
                }
            }
            rk += lo > q0 ? lo - q0 : 0;
        }
        key[u] = k;
        rank[u] = rk < 0 ? 0 : (rk >= n ? n - 1 : rk);
    }
    __syncthreads();   // c is read by the searches above and written by callers next
#pragma unroll
    for (int u = 0; u * kBigThreads < kSmemEntries; ++u) {
        const int i = t + u * kBigThreads;
        if (i >= n) break;
        en.a[rank[u]] = key[u];
        en.b[rank[u]] = i;
    }
    __syncthreads();
}

// record_blocks for a big stripe, one 1024-thread CTA: the stripe's entries
// are stable-sorted by block column, so each run of equal block columns is
// one distinct block with its entries in CSR (= row-major bit) order; the
// run's first entry is the block's first CSR position.  Leaves the sorted
// entries, the run index + 1 of each sorted entry (c) and each run's first
// sorted position (d) for move_values_big.
// in_smem: the scratch is in shared memory (ranked, not sorted); otherwise
// it is the workspace, where build_count_big_kernel left this stripe's
// sorted entry indices (b) and run indices + 1 (c), which are reused.
template <typename I>
__device__ void record_blocks_big(BigShared& sh, const I* indptr, const I* indices, int64_t s, int64_t rows,
                                  int br, int bc, int64_t ncb, const BigEntries& en, uint64_t* code_r,
                                  int64_t* bcol_r, int32_t* first_r, bool in_smem) {
    const int t = threadIdx.x;
    const int64_t r0 = s * br;
    const int64_t r1 = r0 + br < rows ? r0 + br : rows;
    const int64_t e0 = (int64_t)indptr[r0];
    const int n = (int)((int64_t)indptr[r1] - e0);
    if (t <= br) sh.rowstart[t] = (int32_t)((int64_t)indptr[r0 + t < r1 ? r0 + t : r1] - e0);
    if (in_smem && GL_BUILD_SMEM_RANK) {
        __syncthreads();
        big_rank_smem<I>(sh, indices, e0, n, br, bc, ncb * bc, en);
        for (int p = t; p < n; p += kBigThreads) en.c[p] = (p == 0 || en.a[p] != en.a[p - 1]) ? 1 : 0;
        __syncthreads();
        big_scan<false>(sh, en.c, n, true);   // run index + 1
    } else if (!in_smem && GL_BUILD_REUSE_COUNT_SORT) {
        const I* __restrict__ idx = indices + e0;
        const int32_t* __restrict__ b = en.b;
        int32_t* __restrict__ a = en.a;
        for (int p = t; p < n; p += kBigThreads) a[p] = (int32_t)((int64_t)idx[b[p]] / bc);
        __syncthreads();
    } else {
        {   // (restrict pointers scoped to each loop: the arrays are distinct)
            const I* __restrict__ idx = indices + e0;
            int32_t* __restrict__ a = en.a;
            int32_t* __restrict__ b = en.b;
#pragma unroll kUnroll
            for (int i = t; i < n; i += kBigThreads) {
                a[i] = (int32_t)((int64_t)idx[i] / bc);
                b[i] = i;
            }
        }
        __syncthreads();
        const int bits = 64 - __clzll((long long)(ncb > 1 ? ncb - 1 : 1));
        big_sort(sh, en.a, en.b, en.c, en.d, n, bits);
        {
            const int32_t* __restrict__ a = en.a;
            int32_t* __restrict__ c = en.c;
#pragma unroll kUnroll
            for (int p = t; p < n; p += kBigThreads) c[p] = (p == 0 || a[p] != a[p - 1]) ? 1 : 0;
        }
        __syncthreads();
        big_scan<false>(sh, en.c, n, true);   // run index + 1
    }
    {
        const int32_t* __restrict__ a = en.a;
        const int32_t* __restrict__ b = en.b;
        const int32_t* __restrict__ c = en.c;
        int32_t* __restrict__ d = en.d;
        int64_t* __restrict__ bcol = bcol_r;
        int32_t* __restrict__ first = first_r;
        uint64_t* __restrict__ code = code_r;
#pragma unroll kUnroll
        for (int p = t; p < n; p += kBigThreads) {
            if (p == 0 || a[p] != a[p - 1]) {
                const int j = c[p] - 1;
                d[j] = p;
                bcol[j] = a[p];
                first[j] = b[p];
                code[j] = 0;
            }
        }
    }
    __syncthreads();
    {
        const I* __restrict__ idx = indices + e0;
        const int32_t* __restrict__ b = en.b;
        const int32_t* __restrict__ c = en.c;
#pragma unroll kUnroll
        for (int p = t; p < n; p += kBigThreads) {
            const int i = b[p];
            const int r = big_row_of(sh, br, i);
            const int64_t col = (int64_t)idx[i];
            atomicOr(reinterpret_cast<unsigned long long*>(code_r + (c[p] - 1)), 1ull << (r * bc + (int)(col % bc)));
        }
    }
    __syncthreads();
}

// move_values for a big stripe (after record_blocks_big and the ordering):
// kept blocks' entries go straight to block_data at the block's value offset
// plus their rank in the run; the others go to their row's remainder at the
// row's offset plus their rank among the row's dropped entries (an inclusive
// scan of drop flags in CSR order).
template <typename I, typename S>
__device__ void move_values_big(BigShared& sh, const I* indptr, const I* indices, const S* values, int64_t s,
                                int64_t rows, int br, const BigEntries& en, const int32_t* slot,
                                const int32_t* doff, int64_t packed_base, const int64_t* row_rem, S* out_data,
                                I* out_rem_col, S* out_rem_val) {
    const int t = threadIdx.x;
    const int64_t r0 = s * br;
    const int64_t r1 = r0 + br < rows ? r0 + br : rows;
    const int64_t e0 = (int64_t)indptr[r0];
    const int n = (int)((int64_t)indptr[r1] - e0);
    {   // (restrict pointers scoped to each loop: the arrays are distinct)
        const int32_t* __restrict__ b = en.b;
        const int32_t* __restrict__ c = en.c;
        const int32_t* __restrict__ d = en.d;
        const int32_t* __restrict__ sl_r = slot;
        const int32_t* __restrict__ doff_r = doff;
        const S* __restrict__ val = values + e0;
        S* __restrict__ out = out_data + packed_base;
        int32_t* __restrict__ a = en.a;
#pragma unroll kUnroll
        for (int p = t; p < n; p += kBigThreads) {
            const int j = c[p] - 1;
            const int i = b[p];
            const int sl = sl_r[j];
            if (sl >= 0) out[doff_r[j] + (p - d[j])] = val[i];
            a[i] = sl < 0 ? 1 : 0;
        }
    }
    __syncthreads();
    big_scan<false>(sh, en.a, n, true);
    {
        const int32_t* __restrict__ a = en.a;
        const I* __restrict__ idx = indices + e0;
        const S* __restrict__ val = values + e0;
        I* __restrict__ rcol = out_rem_col;
        S* __restrict__ rval = out_rem_val;
#pragma unroll kUnroll
        for (int i = t; i < n; i += kBigThreads) {
            const int32_t before = i > 0 ? a[i - 1] : 0;
            if (a[i] == before) continue;   // kept
            const int r = big_row_of(sh, br, i);
            const int rs = sh.rowstart[r];
            const int32_t row_before = rs > 0 ? a[rs - 1] : 0;
            const int64_t dst = row_rem[r0 + r] + (before - row_before);
            rcol[dst] = idx[i];
            rval[dst] = val[i];
        }
    }
    __syncthreads();
}

// count for a stripe with more than kBigCountEntries entries, one
// 1024-thread CTA: validation of its rows, then a stable sort of its
// entries by block column; runs are the distinct blocks, their codes are
// OR-ed together (two 32-bit halves), and kept blocks, packed values and
// per-row remainder entries are summed.
template <typename I>
__global__ void __launch_bounds__(kBigThreads, GL_BUILD_COUNT_BIG_CTAS)
build_count_big_kernel(const I* indptr, const I* indices, int64_t rows, int64_t cols, int64_t nnz, int br, int bc,
                       int min_nnz, int64_t nstripes, int64_t ncb, BuildWs w) {
    __shared__ BigShared sh;
    extern __shared__ __align__(16) unsigned char build_dyn[];
    __shared__ unsigned long long s_tot[3];   // distinct, kept, packed
    __shared__ int32_t s_rem[33];
    __shared__ int32_t s_bad[3];
    __shared__ int s_item;
    const int t = threadIdx.x;
    for (;;) {
        const int64_t s = list_draw(w.count_list, w.work, kWorkCountHead, nstripes, &s_item);
        if (s < 0) break;
        const int64_t r0 = s * br;
        const int64_t r1 = r0 + br < rows ? r0 + br : rows;
        const int nr = (int)(r1 - r0);
        int64_t e0 = (int64_t)indptr[r0];
        e0 = e0 < 0 ? 0 : (e0 > nnz ? nnz : e0);
        const int n = (int)stripe_entries(indptr, s, rows, nnz, br);
        if (t < 3) {
            s_tot[t] = 0;
            s_bad[t] = 0;
        }
        if (t <= br) s_rem[t] = 0;
        if (t < nr) {   // the rows' indptr
            const int64_t row = r0 + t;
            const int64_t a = (int64_t)indptr[row], b = (int64_t)indptr[row + 1];
            if (a < 0 || b < a || b > nnz || (row == 0 && a != 0) || (row + 1 == rows && b != nnz)) s_bad[kFlagIndptr] = 1;
        }
        if (t <= br) {
            int64_t v = (int64_t)indptr[r0 + t < r1 ? r0 + t : r1] - e0;
            v = v < 0 ? 0 : (v > n ? n : v);
            sh.rowstart[t] = (int32_t)v;
        }
        __syncthreads();
        BigEntries en{w.ent_a + e0, w.ent_b + e0, w.ent_c + e0, w.ent_d + e0};
        if (n <= kSmemEntries) {
            int32_t* d = reinterpret_cast<int32_t*>(build_dyn);
            en = BigEntries{d, d + kSmemEntries, d + 2 * kSmemEntries, d + 3 * kSmemEntries};
        }
        const bool in_smem = n <= kSmemEntries;
        for (int i = t; i < n; i += kBigThreads) {
            int64_t col = (int64_t)indices[e0 + i];
            const int r = big_row_of(sh, br, i);
            if (col < 0 || col >= cols) s_bad[kFlagRange] = 1;
            if (i > sh.rowstart[r] && col <= (int64_t)indices[e0 + i - 1]) s_bad[kFlagNoncanon] = 1;
            col = col < 0 ? 0 : (col >= cols ? cols - 1 : col);
            en.a[i] = (int32_t)(col / bc);
            en.b[i] = i;
        }
        __syncthreads();
        if (in_smem && GL_BUILD_SMEM_RANK) {
            big_rank_smem<I>(sh, indices, e0, n, br, bc, cols, en);
        } else {
            // (the fill reuses b and c of stripes sorted here in the workspace)
            const int bits = 64 - __clzll((long long)(ncb > 1 ? ncb - 1 : 1));
            big_sort(sh, en.a, en.b, en.c, en.d, n, bits);
        }
        for (int p = t; p < n; p += kBigThreads) en.c[p] = (p == 0 || en.a[p] != en.a[p - 1]) ? 1 : 0;
        __syncthreads();
        big_scan<false>(sh, en.c, n, true);   // run index + 1
        const int m = n > 0 ? en.c[n - 1] : 0;
        for (int j = t; j < m; j += kBigThreads) {   // codes: low half in a, high half in d
            en.a[j] = 0;
            en.d[j] = 0;
        }
        __syncthreads();
        for (int p = t; p < n; p += kBigThreads) {
            const int i = en.b[p];
            const int r = big_row_of(sh, br, i);
            int64_t col = (int64_t)indices[e0 + i];
            col = col < 0 ? 0 : (col >= cols ? cols - 1 : col);
            const int bit = r * bc + (int)(col % bc);
            if (bit < 32) atomicOr(reinterpret_cast<unsigned*>(en.a + (en.c[p] - 1)), 1u << bit);
            else atomicOr(reinterpret_cast<unsigned*>(en.d + (en.c[p] - 1)), 1u << (bit - 32));
        }
        __syncthreads();
        for (int j = t; j < m; j += kBigThreads) {
            const int pop = __popc((unsigned)en.a[j]) + __popc((unsigned)en.d[j]);
            atomicAdd(&s_tot[0], 1ull);
            if (pop >= min_nnz) {
                atomicAdd(&s_tot[1], 1ull);
                atomicAdd(&s_tot[2], (unsigned long long)pop);
            }
        }
        for (int p = t; p < n; p += kBigThreads) {
            const int j = en.c[p] - 1;
            const int pop = __popc((unsigned)en.a[j]) + __popc((unsigned)en.d[j]);
            if (pop < min_nnz) atomicAdd(&s_rem[big_row_of(sh, br, en.b[p])], 1);
        }
        __syncthreads();
        if (t == 0) {
            w.stripe_m[s] = (int64_t)s_tot[0];
            w.stripe_kept[s] = (int64_t)s_tot[1];
            w.stripe_packed[s] = (int64_t)s_tot[2];
            if ((int64_t)s_tot[0] > kSmallStripeBlocks)
                list_push(w.fill_list, w.work, kWorkFillHead, nstripes, s, n > kHugeEntries);
            for (int f = 0; f < 3; ++f)
                if (s_bad[f]) atomicOr(&w.flags[f], 1);
        }
        if (t < nr) w.row_rem[r0 + t] = s_rem[t];
        __syncthreads();
    }
}

// order_stripe for a big stripe (one 1024-thread CTA; see the section
// comment above).  Same outputs as order_stripe.
template <typename I>
__device__ void order_stripe_big(BigShared& sh, int64_t s, int m, int n, int br, int bc, int min_nnz, int64_t ncb,
                                 bool key32, int nchain, const int64_t* chain, int64_t prefmax, int64_t kept_base,
                                 int64_t packed_base, const BigRecs& r, uint64_t* out_codes, I* out_coords,
                                 I* out_offsets) {
    const int t = threadIdx.x;
    // Each loop names the distinct record arrays it touches with restrict
    // pointers (scoped to the loop, as list_order_big reaches the same arrays
    // through r), so the compiler keeps several iterations' loads in flight.
    {
        const uint64_t* __restrict__ code = r.code;
        const int32_t* __restrict__ ins = r.ins;
        int32_t* __restrict__ pops = r.pops;
        int32_t* __restrict__ k0 = r.k0;
        int32_t* __restrict__ v0 = r.v0;
#pragma unroll kUnroll
        for (int e = t; e < m; e += kBigThreads) {
            pops[e] = __popcll(code[e]);
            k0[e] = ins[e];
            v0[e] = e;
        }
    }
    __syncthreads();
    // by first CSR position (stripe-local, below n)
    big_sort(sh, r.k0, r.v0, r.k1, r.v1, m, n > 1 ? 32 - __clz(n - 1) : 1);
    {
        int32_t* __restrict__ ins = r.ins;
        const int32_t* __restrict__ v0 = r.v0;
#pragma unroll kUnroll
        for (int i = t; i < m; i += kBigThreads) ins[v0[i]] = i;   // insertion rank
    }
    __syncthreads();
    {
        const int32_t* __restrict__ ins = r.ins;
        int32_t* __restrict__ tau = r.tau;
#pragma unroll kUnroll
        for (int e = t; e < m; e += kBigThreads) tau[e] = ins[e];
    }
    __syncthreads();
    int J = 0;
    while (J + 1 < nchain && chain[2 * (J + 1)] <= prefmax) ++J;
    while (J + 1 < nchain && chain[2 * (J + 1)] <= m) {
        const int present = (int)(chain[2 * (J + 1)] - 1);
        list_order_big(sh, s, ncb, key32, (uint64_t)chain[2 * J + 1], m, present, r);
        {
            const int32_t* __restrict__ ins = r.ins;
            const int32_t* __restrict__ pos = r.pos;
            int32_t* __restrict__ tau = r.tau;
#pragma unroll kUnroll
            for (int e = t; e < m; e += kBigThreads)
                if (ins[e] < present) tau[e] = pos[e];
        }
        __syncthreads();
        ++J;
    }
    list_order_big(sh, s, ncb, key32, (uint64_t)chain[2 * J + 1], m, m, r);
    // kept flags and popcounts in list order; exclusive scans give slots and
    // value offsets
    {
        const int32_t* __restrict__ pops = r.pops;
        const int32_t* __restrict__ pos = r.pos;
        int32_t* __restrict__ k0 = r.k0;
        int32_t* __restrict__ v0 = r.v0;
#pragma unroll kUnroll
        for (int e = t; e < m; e += kBigThreads) {
            const bool kept = pops[e] >= min_nnz;
            k0[pos[e]] = kept ? 1 : 0;
            v0[pos[e]] = kept ? pops[e] : 0;
        }
    }
    __syncthreads();
    big_scan<false>(sh, r.k0, m, false);
    big_scan<false>(sh, r.v0, m, false);
    {
        const uint64_t* __restrict__ code = r.code;
        const int64_t* __restrict__ bcol = r.bcol;
        const int32_t* __restrict__ pops = r.pops;
        const int32_t* __restrict__ pos = r.pos;
        const int32_t* __restrict__ k0 = r.k0;
        const int32_t* __restrict__ v0 = r.v0;
        int32_t* __restrict__ tau = r.tau;
        int32_t* __restrict__ g = r.g;
#pragma unroll kUnroll
        for (int e = t; e < m; e += kBigThreads) {
            int slot = -1, doff = 0;
            if (pops[e] >= min_nnz) {
                slot = k0[pos[e]];
                doff = v0[pos[e]];
                const int64_t ob = kept_base + slot;
                out_codes[ob] = code[e];
                out_coords[2 * ob] = (I)(s * br);
                out_coords[2 * ob + 1] = (I)(bcol[e] * bc);
                out_offsets[ob] = (I)(packed_base + doff);
            }
            tau[e] = slot;
            g[e] = doff;
        }
    }
    __syncthreads();
}

// Emit order and outputs of one stripe's m recorded blocks (team-parallel).
// ins holds first CSR positions on entry.  slot / doff receive, per record,
// the output slot (-1: dropped) and the value offset inside the stripe.
template <int TEAM, typename I>
__device__ void order_stripe(int64_t s, int m, int br, int bc, int min_nnz, int64_t ncb, bool key32, int nchain,
                             const int64_t* chain, int64_t prefmax, int64_t kept_base, int64_t packed_base,
                             const uint64_t* code_r, const int64_t* bcol_r, int32_t* ins, int32_t* tau,
                             uint32_t* bkt, int32_t* g, int32_t* pos, int32_t* pops, uint64_t* out_codes,
                             I* out_coords, I* out_offsets) {
    const int tr = Team<TEAM>::rank();
    for (int e = tr; e < m; e += TEAM) pops[e] = __popcll(code_r[e]);
    // insertion rank = rank of the first CSR position
    for (int e = tr; e < m; e += TEAM) {
        const int32_t fe = ins[e];
        int r = 0;
        for (int f = 0; f < m; ++f) r += ins[f] < fe ? 1 : 0;
        tau[e] = r;
    }
    Team<TEAM>::sync();
    for (int e = tr; e < m; e += TEAM) ins[e] = tau[e];
    Team<TEAM>::sync();
    // bucket count at stripe start, then the rehashes inside the stripe
    int J = 0;
    while (J + 1 < nchain && chain[2 * (J + 1)] <= prefmax) ++J;
    while (J + 1 < nchain && chain[2 * (J + 1)] <= m) {
        const int present = (int)(chain[2 * (J + 1)] - 1);
        list_order<TEAM>(s, ncb, key32, (uint64_t)chain[2 * J + 1], m, present, bcol_r, ins, tau, bkt, g, pos);
        for (int e = tr; e < m; e += TEAM)
            if (ins[e] < present) tau[e] = pos[e];
        Team<TEAM>::sync();
        ++J;
    }
    list_order<TEAM>(s, ncb, key32, (uint64_t)chain[2 * J + 1], m, m, bcol_r, ins, tau, bkt, g, pos);
    // output slot and value offset of each kept block, in list order
    for (int e = tr; e < m; e += TEAM) {
        int slot = -1, doff = 0;
        if (pops[e] >= min_nnz) {
            slot = 0;
            const int32_t pe = pos[e];
            for (int f = 0; f < m; ++f) {
                if (pops[f] >= min_nnz && pos[f] < pe) {
                    ++slot;
                    doff += pops[f];
                }
            }
            const int64_t ob = kept_base + slot;
            out_codes[ob] = code_r[e];
            out_coords[2 * ob] = (I)(s * br);
            out_coords[2 * ob + 1] = (I)(bcol_r[e] * bc);
            out_offsets[ob] = (I)(packed_base + doff);
        }
        tau[e] = slot;
        g[e] = doff;
    }
    Team<TEAM>::sync();
}

// G lanes per stripe (block_rows <= G), 32 / G stripes per warp at a time.
template <typename I, typename S, int G>
__global__ void __launch_bounds__(kBuildThreads)
build_fill_kernel(const I* indptr, const I* indices, const S* values, int64_t rows, int64_t cols, int64_t nnz,
                  int br, int bc, int min_nnz, int64_t nstripes, int64_t ncb, bool key32, int nchain,
                  BuildWs w, uint64_t* out_codes, I* out_coords, I* out_offsets, S* out_data,
                  I* out_rem_col, S* out_rem_val, int32_t* out_stripe_ptr, bool rec) {
    const int lane = threadIdx.x & (G - 1);
    for (WarpDraw<G> d(&w.work[kWorkFillWarpDraw], nstripes); d.next();) {
        const int64_t s = d.s;
        const int64_t rbase = w.stripe_m[s];
        const int m = (int)(w.stripe_m[s + 1] - rbase);
        const int64_t kept_base = w.stripe_kept[s];
        if (lane == 0 && out_stripe_ptr) out_stripe_ptr[s] = (int32_t)kept_base;
        if (m == 0 || m > kSmallStripeBlocks) continue;   // big stripes: build_fill_big_kernel
        if (GL_BUILD_REUSE_COUNT_RECORDS && rec && stripe_entries(indptr, s, rows, nnz, br) <= kBigCountEntries) {
            // the warp count kept this stripe's records
            const int64_t e0 = (int64_t)indptr[s * br];
            for (int j = lane; j < m; j += G) {
                w.rec_code[rbase + j] = (uint64_t)(uint32_t)w.ent_a[e0 + j] | ((uint64_t)(uint32_t)w.ent_b[e0 + j] << 32);
                w.rec_bcol[rbase + j] = w.ent_c[e0 + j];
                w.rec_ins[rbase + j] = w.ent_d[e0 + j];
            }
        } else {
            record_blocks<I, G>(indptr, indices, s, rows, cols, nnz, br, bc, w.rec_code + rbase, w.rec_bcol + rbase,
                                w.rec_ins + rbase);
        }
        __syncwarp(group_mask<G>());
        order_stripe<G, I>(s, m, br, bc, min_nnz, ncb, key32, nchain, w.chain, w.stripe_prefmax[s], kept_base,
                            w.stripe_packed[s], w.rec_code + rbase, w.rec_bcol + rbase, w.rec_ins + rbase,
                            w.rec_tau + rbase, w.rec_bkt + rbase, w.rec_g + rbase, w.rec_pos + rbase,
                            w.rec_pops + rbase, out_codes, out_coords, out_offsets);
        move_values<I, S, G>(indptr, indices, values, s, rows, cols, nnz, br, bc, w.rec_tau + rbase,
                             w.rec_g + rbase, w.stripe_packed[s], w.row_rem, out_data, out_rem_col, out_rem_val);
    }
}

template <typename I, typename S>
__global__ void __launch_bounds__(kBigThreads, GL_BUILD_FILL_BIG_CTAS)
build_fill_big_kernel(const I* indptr, const I* indices, const S* values, int64_t rows, int64_t cols, int64_t nnz,
                      int br, int bc, int min_nnz, int64_t nstripes, int64_t ncb, bool key32, int nchain,
                      BuildWs w, uint64_t* out_codes, I* out_coords, I* out_offsets, S* out_data,
                      I* out_rem_col, S* out_rem_val) {
    __shared__ BigShared sh;
    extern __shared__ __align__(16) unsigned char build_dyn[];
    __shared__ int s_item;
    for (;;) {
        const int64_t s = list_draw(w.fill_list, w.work, kWorkFillHead, nstripes, &s_item);
        if (s < 0) break;
        const int64_t rbase = w.stripe_m[s];
        const int m = (int)(w.stripe_m[s + 1] - rbase);
        const int64_t e0 = (int64_t)indptr[s * br];
        const int64_t r1 = (s + 1) * br < rows ? (s + 1) * br : rows;
        const int64_t n = (int64_t)indptr[r1] - e0;
        BigEntries en{w.ent_a + e0, w.ent_b + e0, w.ent_c + e0, w.ent_d + e0};
        BigRecs r{w.rec_code + rbase, w.rec_bcol + rbase, w.rec_ins + rbase, w.rec_tau + rbase,
                  w.rec_bkt + rbase, w.rec_g + rbase, w.rec_pos + rbase, w.rec_pops + rbase,
                  w.rec_k0 + rbase, w.rec_v0 + rbase, w.rec_k1 + rbase, w.rec_v1 + rbase};
        // m <= n for a CSR the count pass accepted (every block holds an
        // entry); anything else stays on the global scratch, sized by nnz
        const bool in_smem = n >= 0 && n <= kSmemEntries && m <= n;
        if (in_smem) {
            constexpr int K = kSmemEntries;
            uint64_t* d64 = reinterpret_cast<uint64_t*>(build_dyn);
            int32_t* d32 = reinterpret_cast<int32_t*>(d64 + 2 * K);
            en = BigEntries{d32, d32 + K, d32 + 2 * K, d32 + 3 * K};
            int32_t* q = d32 + 4 * K;
            r = BigRecs{d64, reinterpret_cast<int64_t*>(d64 + K), q, q + K, reinterpret_cast<uint32_t*>(q + 2 * K),
                        q + 3 * K, q + 4 * K, q + 5 * K, q + 6 * K, q + 7 * K, q + 8 * K, q + 9 * K};
        }
        record_blocks_big<I>(sh, indptr, indices, s, rows, br, bc, ncb, en, const_cast<uint64_t*>(r.code),
                             const_cast<int64_t*>(r.bcol), r.ins, in_smem);
        order_stripe_big<I>(sh, s, m, (int)n, br, bc, min_nnz, ncb, key32, nchain, w.chain, w.stripe_prefmax[s],
                            w.stripe_kept[s], w.stripe_packed[s], r, out_codes, out_coords, out_offsets);
        move_values_big<I, S>(sh, indptr, indices, values, s, rows, br, en, r.tau, r.g,
                              w.stripe_packed[s], w.row_rem, out_data, out_rem_col, out_rem_val);
    }
}

template <typename I>
__global__ void finish_kernel(const BuildWs w, int64_t rows, int64_t nstripes, I* out_offsets,
                              I* out_rem_indptr, int32_t* out_stripe_ptr) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= rows) out_rem_indptr[i] = (I)w.row_rem[i];
    if (i == 0) {
        out_offsets[w.stripe_kept[nstripes]] = (I)w.stripe_packed[nstripes];
        if (out_stripe_ptr) out_stripe_ptr[nstripes] = (int32_t)w.stripe_kept[nstripes];
        out_offsets[0] = (I)0;
    }
}

int check_args(int32_t index_type, int64_t rows, int64_t cols, int64_t nnz, int32_t br, int32_t bc, int32_t min_nnz) {
    GL_REQUIRE(index_type == GL_I32 || index_type == GL_I64, GL_ERR_INVALID_ARGUMENT, "index_type must be GL_I32 or GL_I64");
    GL_REQUIRE(rows >= 0 && cols >= 0 && nnz >= 0, GL_ERR_INVALID_ARGUMENT, "negative matrix size");
    GL_REQUIRE(br >= 1 && bc >= 1 && (int64_t)br * bc <= 64, GL_ERR_INVALID_ARGUMENT,
               "block_rows * block_cols must be in 1..64 (got %d x %d)", br, bc);
    GL_REQUIRE(br <= 32, GL_ERR_INVALID_ARGUMENT, "block_rows > 32 is not supported by the device builder");
    GL_REQUIRE(ceil_div(rows, br) < (int64_t)(INT32_MAX / 2), GL_ERR_INVALID_ARGUMENT, "too many stripes for int32 stripe lists");
    GL_REQUIRE(min_nnz >= 0 && min_nnz <= 255, GL_ERR_INVALID_ARGUMENT, "min_nnz_per_block must be in 0..255");
    GL_REQUIRE(nnz < (int64_t)INT32_MAX || index_type == GL_I64, GL_ERR_INVALID_ARGUMENT,
               "nnz does not fit the int32 index type");
    return GL_OK;
}

// Bucket counts the standard library's unordered_map goes through when built
// with `hint` buckets and filled one key at a time, as (count, buckets) pairs;
// the first pair is (0, initial buckets).
int bucket_chain_probe(uint64_t hint, int64_t max_elems, int64_t* pairs) {
    std::unordered_map<int64_t, uint8_t> probe(static_cast<size_t>(hint));
    int n = 0;
    size_t last = probe.bucket_count();
    pairs[0] = 0;
    pairs[1] = (int64_t)last;
    n = 1;
    for (int64_t i = 0; i < max_elems; ++i) {
        probe.emplace(i, 0);
        if (probe.bucket_count() != last) {
            last = probe.bucket_count();
            if (n >= kMaxChain) return -1;
            pairs[2 * n] = i + 1;
            pairs[2 * n + 1] = (int64_t)last;
            ++n;
        }
    }
    return n;
}

// bucket_chain_probe, remembered per hint: the chain for fewer elements is a
// prefix of the chain for more, so the longest one probed so far answers
// every request up to its length (a 17 k-element probe costs the host about
// a millisecond per build otherwise).
int bucket_chain(uint64_t hint, int64_t max_elems, int64_t* pairs) {
    struct Chain {
        int64_t upto = -1;
        int n = 0;
        int64_t pairs[2 * kMaxChain];
    };
    static std::unordered_map<uint64_t, Chain> cache;
    std::lock_guard<std::mutex> lock(setup_mutex());
    Chain& c = cache[hint];
    if (c.upto < max_elems) {
        const int n = bucket_chain_probe(hint, max_elems, c.pairs);
        if (n < 0) {
            c.upto = -1;
            return -1;
        }
        c.n = n;
        c.upto = max_elems;
    }
    int n = 0;
    while (n < c.n && c.pairs[2 * n] <= max_elems) {
        pairs[2 * n] = c.pairs[2 * n];
        pairs[2 * n + 1] = c.pairs[2 * n + 1];
        ++n;
    }
    return n;
}

template <typename I>
int count_impl(const I* indptr, const I* indices, int64_t rows, int64_t cols, int64_t nnz, int32_t br, int32_t bc,
               int32_t min_nnz, const BuildWs& w, gl_pbr_build_counts* counts, cudaStream_t stream) {
    const int64_t ns = ceil_div(rows, br);
    GL_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int32_t) * kNumFlags, stream));
    GL_CUDA_TRY(cudaMemsetAsync(w.work, 0, sizeof(int32_t) * kNumWork, stream));
    {
        // The trailing slot of every count array must be zero for the scans.
        int64_t* regions[5] = {w.stripe_m, w.stripe_kept, w.stripe_packed, w.stripe_prefmax, w.row_rem};
        const int64_t lens[5] = {ns + 1, ns + 1, ns + 1, ns + 1, rows + 1};
        for (int i = 0; i < 5; ++i) GL_CUDA_TRY(cudaMemsetAsync(regions[i], 0, 8 * lens[i], stream));
    }
    if (ns > 0) {
        int64_t blocks = ceil_div(ns, kBuildWarps);
        const int64_t cap = (int64_t)num_sms() * 16;
        if (blocks > cap) blocks = cap;
#ifndef GL_BUILD_COUNT_GROUP
#define GL_BUILD_COUNT_GROUP 8
#endif
        const bool rec = ceil_div(cols, bc) < (int64_t)INT32_MAX;   // block columns fit the int32 records
        if (br <= 8 && GL_BUILD_COUNT_GROUP <= 8)
            build_count_kernel<I, 8><<<(unsigned)blocks, kBuildThreads, 0, stream>>>(indptr, indices, rows, cols, nnz,
                                                                                     br, bc, min_nnz, ns, w, rec);
        else if (br <= 16 && GL_BUILD_COUNT_GROUP <= 16)
            build_count_kernel<I, 16><<<(unsigned)blocks, kBuildThreads, 0, stream>>>(indptr, indices, rows, cols,
                                                                                      nnz, br, bc, min_nnz, ns, w, rec);
        else
            build_count_kernel<I, 32><<<(unsigned)blocks, kBuildThreads, 0, stream>>>(indptr, indices, rows, cols,
                                                                                      nnz, br, bc, min_nnz, ns, w, rec);
        GL_LAUNCH_CHECK("build_count_kernel");
        const int64_t ncb = ceil_div(cols, bc);
        int64_t big_blocks = (int64_t)num_sms() * GL_BUILD_COUNT_BIG_CTAS;
        if (big_blocks > ns) big_blocks = ns;
        static std::atomic<int> attr_cache[kMaxDevices];
        int attr = 0;
        const int arc = per_device_value(
            attr_cache,
            [&](int* v) {
                GL_CUDA_TRY(cudaFuncSetAttribute(build_count_big_kernel<I>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 kCountSmemBytes));
                *v = 1;
                return GL_OK;
            },
            &attr);
        if (arc != GL_OK) return arc;
        build_count_big_kernel<I><<<(unsigned)big_blocks, kBigThreads, kCountSmemBytes, stream>>>(
            indptr, indices, rows, cols, nnz, br, bc, min_nnz, ns, ncb, w);
        GL_LAUNCH_CHECK("build_count_big_kernel");
    }
    int rc;
    // exclusive running max of distinct blocks per stripe (bucket state)
    if ((rc = exclusive_scan<int64_t, OpMax>(w.stripe_m, w.stripe_prefmax, ns + 1, w.scan_scratch, int64_t(0),
                                             OpMax(), stream)) != GL_OK)
        return rc;
    if ((rc = exclusive_scan<int64_t, OpSum>(w.stripe_m, w.stripe_m, ns + 1, w.scan_scratch, int64_t(0), OpSum(),
                                             stream)) != GL_OK)
        return rc;
    if ((rc = exclusive_scan<int64_t, OpSum>(w.stripe_kept, w.stripe_kept, ns + 1, w.scan_scratch, int64_t(0),
                                             OpSum(), stream)) != GL_OK)
        return rc;
    if ((rc = exclusive_scan<int64_t, OpSum>(w.stripe_packed, w.stripe_packed, ns + 1, w.scan_scratch, int64_t(0),
                                             OpSum(), stream)) != GL_OK)
        return rc;
    if ((rc = exclusive_scan<int64_t, OpSum>(w.row_rem, w.row_rem, rows + 1, w.scan_scratch, int64_t(0), OpSum(),
                                             stream)) != GL_OK)
        return rc;
    int32_t flags[kNumFlags];
    int64_t tot[5];
    GL_CUDA_TRY(cudaMemcpyAsync(flags, w.flags, sizeof(flags), cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaMemcpyAsync(&tot[0], w.stripe_kept + ns, 8, cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaMemcpyAsync(&tot[1], w.stripe_packed + ns, 8, cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaMemcpyAsync(&tot[2], w.row_rem + rows, 8, cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaMemcpyAsync(&tot[3], w.stripe_prefmax + ns, 8, cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaMemcpyAsync(&tot[4], w.stripe_m + ns, 8, cudaMemcpyDeviceToHost, stream));
    GL_CUDA_TRY(cudaStreamSynchronize(stream));
    GL_REQUIRE(!flags[kFlagIndptr], GL_ERR_INVALID_ARGUMENT,
               "CSR indptr must start at 0, be non-decreasing and end at nnz=%lld", (long long)nnz);
    GL_REQUIRE(!flags[kFlagRange], GL_ERR_INVALID_ARGUMENT, "CSR column index out of range [0, %lld)",
               (long long)cols);
    GL_REQUIRE(!flags[kFlagNoncanon], GL_ERR_NONCANONICAL,
               "CSR rows must have strictly increasing column indices (sorted, no duplicates)");
    GL_REQUIRE(tot[0] + tot[2] <= nnz && tot[1] + tot[2] == nnz, GL_ERR_INVALID_ARGUMENT,
               "CSR indptr does not describe nnz=%lld entries", (long long)nnz);
    GL_REQUIRE(tot[0] < (int64_t)INT32_MAX, GL_ERR_INVALID_ARGUMENT, "too many blocks for int32 stripe pointers");
    counts->num_blocks = tot[0];
    counts->packed_nnz = tot[1];
    counts->remainder_nnz = tot[2];
    counts->max_stripe_blocks = tot[3];
    counts->distinct_blocks = tot[4];
    return GL_OK;
}

template <typename I, typename S>
int fill_impl(const I* indptr, const I* indices, const S* values, int64_t rows, int64_t cols, int64_t nnz, int32_t br,
              int32_t bc,
              int32_t min_nnz, const BuildWs& w, const gl_pbr_build_counts* counts, uint64_t* codes, I* coords,
              I* offsets, S* data, I* rem_indptr, I* rem_col, S* rem_val, int32_t* stripe_ptr, cudaStream_t stream) {
    const int64_t ns = ceil_div(rows, br);
    const uint64_t ncb = (uint64_t)ceil_div(cols, bc);
    const uint64_t hint = (uint64_t)std::sqrt((double)ncb);
    int64_t chain[2 * kMaxChain];
    const int nchain = bucket_chain(hint, counts->max_stripe_blocks, chain);
    GL_REQUIRE(nchain > 0, GL_ERR_INVALID_ARGUMENT, "bucket chain longer than %d steps", kMaxChain);
    GL_CUDA_TRY(cudaMemcpyAsync(w.chain, chain, sizeof(int64_t) * 2 * nchain, cudaMemcpyHostToDevice, stream));
    if (ns > 0) {
        // the fill's draw counters are reset here, so a fill may be repeated after one count
        GL_CUDA_TRY(cudaMemsetAsync(w.work + kWorkFillDraw, 0, 2 * sizeof(int32_t), stream));
        int64_t blocks = ceil_div(ns, kBuildWarps);
        const int64_t cap = (int64_t)num_sms() * 16;
        if (blocks > cap) blocks = cap;
#ifndef GL_BUILD_FILL_GROUP
#define GL_BUILD_FILL_GROUP 8
#endif
#define GL_FILL_LAUNCH(G)                                                                                        \
    build_fill_kernel<I, S, G><<<(unsigned)blocks, kBuildThreads, 0, stream>>>(                                   \
        indptr, indices, values, rows, cols, nnz, br, bc, min_nnz, ns, (int64_t)ncb, sizeof(I) == 4, nchain, w,   \
        codes, coords, offsets, data, rem_col, rem_val, stripe_ptr, ncb < (uint64_t)INT32_MAX)
        if (br <= 8 && GL_BUILD_FILL_GROUP <= 8) GL_FILL_LAUNCH(8);
        else if (br <= 16 && GL_BUILD_FILL_GROUP <= 16) GL_FILL_LAUNCH(16);
        else GL_FILL_LAUNCH(32);
#undef GL_FILL_LAUNCH
        GL_LAUNCH_CHECK("build_fill_kernel");
        if (counts->max_stripe_blocks > kSmallStripeBlocks) {
            int64_t big_blocks = (int64_t)num_sms() * GL_BUILD_FILL_BIG_CTAS;
            if (big_blocks > ns) big_blocks = ns;
            static std::atomic<int> attr_cache[kMaxDevices];
            int attr = 0;
            const int arc = per_device_value(
                attr_cache,
                [&](int* v) {
                    GL_CUDA_TRY(cudaFuncSetAttribute(build_fill_big_kernel<I, S>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, kFillSmemBytes));
                    *v = 1;
                    return GL_OK;
                },
                &attr);
            if (arc != GL_OK) return arc;
            build_fill_big_kernel<I, S><<<(unsigned)big_blocks, kBigThreads, kFillSmemBytes, stream>>>(
                indptr, indices, values, rows, cols, nnz, br, bc, min_nnz, ns, (int64_t)ncb, sizeof(I) == 4, nchain,
                w, codes, coords, offsets, data, rem_col, rem_val);
            GL_LAUNCH_CHECK("build_fill_big_kernel");
        }
    }
    finish_kernel<I><<<(unsigned)ceil_div(rows + 1, 256), 256, 0, stream>>>(w, rows, ns, offsets, rem_indptr,
                                                                            stripe_ptr);
    GL_LAUNCH_CHECK("finish_kernel");
    // The chain lives in host stack memory: make sure the copy finished.
    GL_CUDA_TRY(cudaStreamSynchronize(stream));
    return GL_OK;
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int64_t gl_pbr_build_workspace_bytes(int64_t rows, int64_t cols, int64_t nnz, int32_t block_rows,
                                                int32_t block_cols) {
    (void)cols;
    (void)block_cols;
    if (rows < 0 || nnz < 0 || block_rows < 1) return -1;
    return layout_ws(nullptr, rows, nnz, block_rows).bytes;
}

extern "C" int gl_pbr_build_count(const void* indptr, const void* indices, int32_t index_type, int64_t rows,
                                  int64_t cols, int64_t nnz, int32_t block_rows, int32_t block_cols,
                                  int32_t min_nnz_per_block, void* workspace, int64_t workspace_bytes,
                                  gl_pbr_build_counts* counts, cudaStream_t stream) {
    int rc = check_args(index_type, rows, cols, nnz, block_rows, block_cols, min_nnz_per_block);
    if (rc != GL_OK) return rc;
    GL_REQUIRE(counts != nullptr, GL_ERR_INVALID_ARGUMENT, "counts is NULL");
    const BuildWs w = layout_ws(workspace, rows, nnz, block_rows);
    GL_REQUIRE(workspace != nullptr && workspace_bytes >= w.bytes, GL_ERR_WORKSPACE,
               "workspace of %lld bytes needed", (long long)w.bytes);
    GL_REQUIRE(rows == 0 || indptr != nullptr, GL_ERR_INVALID_ARGUMENT, "indptr is NULL");
    if (index_type == GL_I32)
        return count_impl<int32_t>(static_cast<const int32_t*>(indptr), static_cast<const int32_t*>(indices), rows,
                                   cols, nnz, block_rows, block_cols, min_nnz_per_block, w, counts, stream);
    return count_impl<int64_t>(static_cast<const int64_t*>(indptr), static_cast<const int64_t*>(indices), rows, cols,
                               nnz, block_rows, block_cols, min_nnz_per_block, w, counts, stream);
}

extern "C" int gl_pbr_build_fill(const void* indptr, const void* indices, const void* values, int32_t index_type,
                                 int32_t value_type, int64_t rows, int64_t cols, int64_t nnz, int32_t block_rows,
                                 int32_t block_cols, int32_t min_nnz_per_block, void* workspace,
                                 int64_t workspace_bytes, const gl_pbr_build_counts* counts, uint64_t* block_codes,
                                 void* block_coords, void* block_offsets, void* block_data, void* remainder_indptr,
                                 void* remainder_col_ind, void* remainder_data, int32_t* stripe_block_ptr,
                                 cudaStream_t stream) {
    int rc = check_args(index_type, rows, cols, nnz, block_rows, block_cols, min_nnz_per_block);
    if (rc != GL_OK) return rc;
    GL_REQUIRE(value_type == GL_F32 || value_type == GL_F64, GL_ERR_INVALID_ARGUMENT, "value_type must be GL_F32 or GL_F64");
    GL_REQUIRE(counts != nullptr, GL_ERR_INVALID_ARGUMENT, "counts is NULL");
    const BuildWs w = layout_ws(workspace, rows, nnz, block_rows);
    GL_REQUIRE(workspace != nullptr && workspace_bytes >= w.bytes, GL_ERR_WORKSPACE,
               "workspace of %lld bytes needed", (long long)w.bytes);
    GL_REQUIRE(block_offsets != nullptr && remainder_indptr != nullptr, GL_ERR_INVALID_ARGUMENT,
               "block_offsets / remainder_indptr are NULL");
#define GL_FILL(I, S)                                                                                             \
    return fill_impl<I, S>(static_cast<const I*>(indptr), static_cast<const I*>(indices),                         \
                           static_cast<const S*>(values), rows, cols, nnz, block_rows, block_cols, min_nnz_per_block, w, \
                           counts, block_codes, static_cast<I*>(block_coords), static_cast<I*>(block_offsets),    \
                           static_cast<S*>(block_data), static_cast<I*>(remainder_indptr),                       \
                           static_cast<I*>(remainder_col_ind), static_cast<S*>(remainder_data), stripe_block_ptr, \
                           stream)
    if (index_type == GL_I32) {
        if (value_type == GL_F32) GL_FILL(int32_t, float);
        GL_FILL(int32_t, double);
    }
    if (value_type == GL_F32) GL_FILL(int64_t, float);
    GL_FILL(int64_t, double);
#undef GL_FILL
}
