// FP32 instances of the fused stripe kernel (SpMM and power-iteration step).
#include "stripe_launch.cuh"
#include "window_kernel.cuh"

namespace gl {

namespace {
template <bool PPR, int BR>
int dispatch_f32(const StripeArgs<float>& a, int tile_hint, int lane_split, cudaStream_t st) {
    // the half-warp shape is register-heavy with the power-iteration
    // epilogue, so only the plain SpMM uses it
    if constexpr (!PPR) {
        // the window kernel (staged X windows) when asked for and its shape
        // applies (no other column tile / lane split)
        if (a.variant == 2 && tile_hint <= 0 && lane_split == 0 && window_eligible(a)) return launch_window<BR>(a, st);
    }
    const Shape sh = pick_shape<float>(a.K, tile_hint, a.X, a.Y, !PPR, lane_split);
    if constexpr (!PPR) {
        if (sh.V == 4 && sh.C == 16) return launch_stripe_shape<float, BR, 4, 16, PPR>(a, st);
    }
    switch (sh.V * 100 + sh.C) {
        case 432: return launch_stripe_shape<float, BR, 4, 32, PPR>(a, st);
        case 232: return launch_stripe_shape<float, BR, 2, 32, PPR>(a, st);
        case 132: return launch_stripe_shape<float, BR, 1, 32, PPR>(a, st);
        case 116: return launch_stripe_shape<float, BR, 1, 16, PPR>(a, st);
        case 108: return launch_stripe_shape<float, BR, 1, 8, PPR>(a, st);
        case 104: return launch_stripe_shape<float, BR, 1, 4, PPR>(a, st);
        case 102: return launch_stripe_shape<float, BR, 1, 2, PPR>(a, st);
        default: return launch_stripe_shape<float, BR, 1, 1, PPR>(a, st);
    }
}
}  // namespace

template <bool PPR>
static int launch_f32(const StripeArgs<float>& a, int br, int bc, int tile_hint, int lane_split, cudaStream_t st) {
    if (br == 2 && bc == 2) return dispatch_f32<PPR, 2>(a, tile_hint, lane_split, st);
    if (br == 4 && bc == 4) return dispatch_f32<PPR, 4>(a, tile_hint, lane_split, st);
    if (br == 8 && bc == 8) return dispatch_f32<PPR, 8>(a, tile_hint, lane_split, st);
    set_error("Unsupported block size for PBR SpMM. Only 2x2, 4x4, and 8x8 are supported.");
    return GL_ERR_UNSUPPORTED_BLOCK;
}

template <>
int launch_stripe<float, false>(const StripeArgs<float>& a, int br, int bc, int tile_hint, int lane_split,
                            cudaStream_t st) {
    return launch_f32<false>(a, br, bc, tile_hint, lane_split, st);
}
template <>
int launch_stripe<float, true>(const StripeArgs<float>& a, int br, int bc, int tile_hint, int lane_split,
                            cudaStream_t st) {
    return launch_f32<true>(a, br, bc, tile_hint, lane_split, st);
}

}  // namespace gl
