// Oracle — test infrastructure only.  Nothing in the product links or loads
// this file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// use it as the checker for the GPU PBR builder.
//
// CPU restatement of the reference PBR builder `csr_to_pbr<index_t, scalar_t>`
// (Backend/graph_link/pbr_matrix/pbr_matrix.cpp:340-477), written as plain
// C-ABI functions over arrays so that ctypes can call them.
//
// What has to be identical to the reference, and why:
//   * the stripe walk: rows are consumed in order; a stripe (a row of blocks)
//     is closed when (row + 1) / block_rows moves past the current block row
//     (pbr_matrix.cpp:399-401), and the trailing partial stripe is closed after
//     the loop (pbr_matrix.cpp:431-452);
//   * the emit order of the blocks of a stripe is the iteration order of a
//     std::unordered_map keyed by the block index truncated to index_t, built
//     with a bucket hint of sqrt(number of column blocks) and cleared (not
//     destroyed) between stripes (pbr_matrix.cpp:374-376, 389, 402, 425).
//     That order is part of the reference's observable output, so the oracle
//     reproduces it with the same standard-library container;
//   * keep rule: popcount(code) >= min_nnz_per_block (pbr_matrix.cpp:403-404);
//   * a kept block appends every value routed to it in CSR order and advances
//     the offset by popcount (pbr_matrix.cpp:405-412);
//   * a dropped block hands its k-th routed value to its k-th set bit in bit
//     order (pbr_matrix.cpp:413-422), and each remainder row is sorted by
//     (column, value) (pbr_matrix.cpp:455-458).
//
// Build: g++ -O2 -std=c++17 -shared -fPIC oracle/pbr_oracle.cpp -o <out>.so
// (oracle.build_oracle() in oracle/__init__.py does this).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <utility>
#include <vector>

namespace {

template <typename I, typename S>
struct OraclePbr {
    int64_t rows = 0, cols = 0, block_rows = 0, block_cols = 0, total_nnz = 0;
    std::vector<uint64_t> codes;
    std::vector<I> coords;        // flat [row0, col0, row1, col1, ...]
    std::vector<I> offsets;       // nb + 1
    std::vector<S> data;
    std::vector<I> rem_indptr;    // rows + 1
    std::vector<I> rem_col;
    std::vector<S> rem_val;
};

// One open block of the stripe being assembled.
template <typename I, typename S>
struct OpenBlock {
    uint64_t code = 0;
    I row0 = 0, col0 = 0;
    std::vector<S> vals;          // values in the order they were routed here
};

template <typename I, typename S>
OraclePbr<I, S>* build(const I* indptr, const I* indices, const S* vals,
                       int64_t rows, int64_t cols, int64_t br, int64_t bc,
                       int min_nnz) {
    auto* out = new OraclePbr<I, S>();
    out->rows = rows; out->cols = cols; out->block_rows = br; out->block_cols = bc;
    out->total_nnz = rows > 0 ? static_cast<int64_t>(indptr[rows]) : 0;

    const uint64_t n_col_blocks = (static_cast<uint64_t>(cols) + bc - 1) / bc;
    // Same hint expression as the reference: sqrt of an unsigned 64-bit count,
    // converted to the container's size_type.
    std::unordered_map<I, size_t> slot_of(
        static_cast<size_t>(std::sqrt(static_cast<double>(n_col_blocks))));
    std::vector<OpenBlock<I, S>> open;
    std::vector<std::vector<std::pair<I, S>>> rem_rows(rows);
    int64_t running = 0;
    out->offsets.push_back(0);

    auto close_stripe = [&]() {
        for (const auto& kv : slot_of) {
            OpenBlock<I, S>& b = open[kv.second];
            const int pop = __builtin_popcountll(b.code);
            if (pop >= min_nnz) {
                out->codes.push_back(b.code);
                out->coords.push_back(b.row0);
                out->coords.push_back(b.col0);
                out->data.insert(out->data.end(), b.vals.begin(), b.vals.end());
                running += pop;
                out->offsets.push_back(static_cast<I>(running));
            } else {
                size_t k = 0;
                for (int64_t bit = 0; bit < br * bc; ++bit) {
                    if ((b.code >> bit) & 1ull) {
                        rem_rows[b.row0 + bit / bc].emplace_back(
                            static_cast<I>(b.col0 + bit % bc), b.vals[k++]);
                    }
                }
            }
        }
        slot_of.clear();
        open.clear();
    };

    for (int64_t row = 0; row < rows; ++row) {
        const uint64_t brow = static_cast<uint64_t>(row) / br;
        const uint64_t r_in = static_cast<uint64_t>(row) % br;
        for (int64_t j = indptr[row]; j < static_cast<int64_t>(indptr[row + 1]); ++j) {
            const uint64_t col = static_cast<uint64_t>(indices[j]);
            const uint64_t bcol = col / bc;
            const I key = static_cast<I>(brow * n_col_blocks + bcol);
            auto ins = slot_of.emplace(key, open.size());
            if (ins.second) {
                OpenBlock<I, S> nb;
                nb.row0 = static_cast<I>(brow * br);
                nb.col0 = static_cast<I>(bcol * bc);
                open.push_back(std::move(nb));
            }
            OpenBlock<I, S>& b = open[ins.first->second];
            b.code |= 1ull << (r_in * bc + col % bc);
            b.vals.push_back(vals[j]);
        }
        if (static_cast<uint64_t>(row + 1) / br > brow) close_stripe();
    }
    close_stripe();  // trailing partial stripe (no-op when rows % br == 0)

    out->rem_indptr.assign(rows + 1, 0);
    for (int64_t r = 0; r < rows; ++r) {
        std::sort(rem_rows[r].begin(), rem_rows[r].end());
        out->rem_indptr[r + 1] = out->rem_indptr[r] + static_cast<I>(rem_rows[r].size());
        for (const auto& cv : rem_rows[r]) {
            out->rem_col.push_back(cv.first);
            out->rem_val.push_back(cv.second);
        }
    }
    return out;
}

template <typename T>
void copy_out(const std::vector<T>& v, T* dst) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}

}  // namespace

#define GL_ORACLE_DEFINE(SUFFIX, I, S)                                                      \
    extern "C" void* oracle_csr_to_pbr_##SUFFIX(const I* indptr, const I* indices,          \
                                                const S* vals, int64_t rows, int64_t cols,  \
                                                int64_t br, int64_t bc, int min_nnz) {      \
        return build<I, S>(indptr, indices, vals, rows, cols, br, bc, min_nnz);             \
    }                                                                                       \
    extern "C" void oracle_pbr_sizes_##SUFFIX(const void* h, int64_t* out4) {               \
        auto* m = static_cast<const OraclePbr<I, S>*>(h);                                   \
        out4[0] = static_cast<int64_t>(m->codes.size());                                    \
        out4[1] = static_cast<int64_t>(m->data.size());                                     \
        out4[2] = static_cast<int64_t>(m->rem_col.size());                                  \
        out4[3] = m->total_nnz;                                                             \
    }                                                                                       \
    extern "C" void oracle_pbr_copy_##SUFFIX(const void* h, uint64_t* codes, I* coords,     \
                                             I* offsets, S* data, I* rem_indptr,            \
                                             I* rem_col, S* rem_val) {                      \
        auto* m = static_cast<const OraclePbr<I, S>*>(h);                                   \
        copy_out(m->codes, codes); copy_out(m->coords, coords);                             \
        copy_out(m->offsets, offsets); copy_out(m->data, data);                             \
        copy_out(m->rem_indptr, rem_indptr); copy_out(m->rem_col, rem_col);                 \
        copy_out(m->rem_val, rem_val);                                                      \
    }                                                                                       \
    extern "C" void oracle_pbr_free_##SUFFIX(void* h) {                                     \
        delete static_cast<OraclePbr<I, S>*>(h);                                            \
    }

GL_ORACLE_DEFINE(i32_f32, int32_t, float)
GL_ORACLE_DEFINE(i32_f64, int32_t, double)
GL_ORACLE_DEFINE(i64_f32, int64_t, float)
GL_ORACLE_DEFINE(i64_f64, int64_t, double)

// Bucket counts the standard library's unordered_map goes through when it is
// built with a hint and filled one key at a time (the container the reference
// keys its stripes by).  Writes up to `cap` pairs (element count that triggered
// the change, new bucket count); the first pair is (0, initial bucket count).
extern "C" int64_t oracle_bucket_chain(uint64_t hint, int64_t max_elems, int64_t* out_pairs,
                                       int64_t cap) {
    std::unordered_map<int64_t, uint8_t> m(static_cast<size_t>(hint));
    int64_t n = 0;
    size_t last = m.bucket_count();
    if (n < cap) { out_pairs[2 * n] = 0; out_pairs[2 * n + 1] = static_cast<int64_t>(last); ++n; }
    for (int64_t i = 0; i < max_elems; ++i) {
        m.emplace(i, 0);
        if (m.bucket_count() != last) {
            last = m.bucket_count();
            if (n < cap) { out_pairs[2 * n] = i + 1; out_pairs[2 * n + 1] = static_cast<int64_t>(last); ++n; }
        }
    }
    return n;
}
