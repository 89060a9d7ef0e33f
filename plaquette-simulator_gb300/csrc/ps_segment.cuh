// ps_segment.cuh -- device-side structures of compiled circuits.
#pragma once
#include "ps_common.cuh"

namespace ps {

// Per-run parameters read by every kernel of a compiled circuit, so one
// captured CUDA graph can be replayed with a new seed / event base.
struct RunParams {
    uint64_t seed;
    uint64_t event_base;
};

// A gate inside a fused segment.  a / b are LOCAL column indices (positions
// in the segment's touched-qubit list); rec indexes the record table for the
// per-shot conditional gates.
struct SegGate {
    int32_t code;
    int32_t a;
    int32_t b;
    int32_t rec;
};

// A sign operation r ^= (fx & z_a) ^ (fz & x_a): the Pauli gates (constant
// masks, GateFunctors.hpp:303-307,323-327,372-376) and the X of a reset
// (mask = record outcome).
enum SignKind : int32_t { SIGN_X = 0, SIGN_Y = 1, SIGN_Z = 2, SIGN_REC_X = 3 };
struct SegSign {
    int32_t kind;
    int32_t a;
    int32_t rec;
    int32_t pad;
};

// Layer L: gates [g0, g1) act on disjoint columns; afterwards sign ops
// [s0, s1) and the noise entries tagged with layer L.
struct SegLayer {
    int32_t g0, g1, s0, s1;
};

// One Pauli channel of a segment.  thr_off indexes the threshold table
// (3 or 15 entries); event is the op's event offset within the run.
struct NoiseSlot {
    int32_t layer;
    int32_t a;   // local column
    int32_t b;   // local column or -1
    int32_t count;  // 3 or 15
    int32_t thr_off;
    uint32_t event;
};

// Sampled channel outcome for one 64-shot word: X/Z components on a and b.
struct NoiseEntry {
    u64 fxa, fza, fxb, fzb;
    int32_t slot;
    int32_t layer;
};

struct SegmentDev {
    const SegLayer *layers;
    int32_t nlayers;
    const SegGate *gates;
    const SegSign *signs;
    const int32_t *cols;     // touched global qubits, nq entries
    int32_t nq;
    const NoiseSlot *slots;
    int32_t nslots;
    const uint64_t *thr;     // threshold table
    NoiseEntry *entries;     // [w][cap]
    int32_t *entry_count;    // [w]
    int32_t cap;
    u64 *dense;              // [w][nslots][4] sampling scratch
};

}  // namespace ps
