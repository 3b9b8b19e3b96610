// FP64 instances of the fused stripe kernel (the reference's PBRMatrix*Double
// path; a compatibility path, not a tuned one).
#include "stripe_launch.cuh"

namespace gl {

namespace {
template <bool PPR, int BR>
int dispatch_f64(const StripeArgs<double>& a, int tile_hint, int lane_split, cudaStream_t st) {
    const Shape sh = pick_shape<double>(a.K, tile_hint, a.X, a.Y, false, lane_split);
    if (sh.C == 32 && sh.V == 2) return launch_stripe_shape<double, BR, 2, 32, PPR>(a, st);
    if (sh.C == 32) return launch_stripe_shape<double, BR, 1, 32, PPR>(a, st);
    return launch_stripe_shape<double, BR, 1, 1, PPR>(a, st);
}
}  // namespace

template <bool PPR>
static int launch_f64(const StripeArgs<double>& a, int br, int bc, int tile_hint, int lane_split, cudaStream_t st) {
    if (br == 2 && bc == 2) return dispatch_f64<PPR, 2>(a, tile_hint, lane_split, st);
    if (br == 4 && bc == 4) return dispatch_f64<PPR, 4>(a, tile_hint, lane_split, st);
    if (br == 8 && bc == 8) return dispatch_f64<PPR, 8>(a, tile_hint, lane_split, st);
    set_error("Unsupported block size for PBR SpMM. Only 2x2, 4x4, and 8x8 are supported.");
    return GL_ERR_UNSUPPORTED_BLOCK;
}

template <>
int launch_stripe<double, false>(const StripeArgs<double>& a, int br, int bc, int tile_hint, int lane_split,
                            cudaStream_t st) {
    return launch_f64<false>(a, br, bc, tile_hint, lane_split, st);
}
template <>
int launch_stripe<double, true>(const StripeArgs<double>& a, int br, int bc, int tile_hint, int lane_split,
                            cudaStream_t st) {
    return launch_f64<true>(a, br, bc, tile_hint, lane_split, st);
}

}  // namespace gl
