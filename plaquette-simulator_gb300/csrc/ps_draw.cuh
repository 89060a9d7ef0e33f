// ps_draw.cuh -- the random outcome of a measurement for the 64 shots of
// one word (MeasureRandom's `frand(0,1) < bias`, MeasurementFunctors.hpp:
// 225-265, with a Philox draw or a forced bit), shared by the per-shot and
// shared-x/z measurement kernels so both draw identically.
#pragma once
#include "ps_internal.h"

namespace ps {

// k: the state's word; the draw is keyed by the global word word_base + k.
__device__ __forceinline__ u64 outcome_bits(const MeasOp &op, int lane, uint64_t seed, uint64_t event_base,
                                            int64_t k, uint64_t word_base) {
    u64 bits = 0ull;
    if (lane < 16) {
        if (op.forced) {
            const u64 fw = op.forced[k];
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const int b = lane * 4 + l;
                const float u = ((fw >> b) & 1ull) ? 0.25f : 0.75f;
                if (u < op.bias) bits |= 1ull << b;
            }
        } else {
            const u32x4 u =
                draw_block(seed, event_base + op.event, word_base + (uint64_t)k, (uint32_t)lane, TAG_MEASURE);
#pragma unroll
            for (int l = 0; l < 4; ++l)
                if (unit_float(u.v[l]) < op.bias) bits |= 1ull << (lane * 4 + l);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) bits |= __shfl_xor_sync(0xffffffffu, bits, off);
    return bits;
}

// The same 64 outcomes computed by one thread (all 16 Philox blocks).
__device__ __forceinline__ u64 outcome_word(const MeasOp &op, uint64_t seed, uint64_t event_base, int64_t k,
                                            uint64_t word_base) {
    u64 bits = 0ull;
    if (op.forced) {
        const u64 fw = op.forced[k];
        for (int b = 0; b < 64; ++b) {
            const float u = ((fw >> b) & 1ull) ? 0.25f : 0.75f;
            if (u < op.bias) bits |= 1ull << b;
        }
        return bits;
    }
    for (uint32_t sub = 0; sub < 16; ++sub) {
        const u32x4 u = draw_block(seed, event_base + op.event, word_base + (uint64_t)k, sub, TAG_MEASURE);
#pragma unroll
        for (int l = 0; l < 4; ++l)
            if (unit_float(u.v[l]) < op.bias) bits |= 1ull << (sub * 4 + l);
    }
    return bits;
}

}  // namespace ps
