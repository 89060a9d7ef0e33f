// ps_segment.cuh -- device-side structures of compiled circuits.
#pragma once
#include "ps_common.cuh"

namespace ps {

// Per-run parameters read by every kernel of a compiled circuit, so one
// captured CUDA graph can be replayed with a new seed / event base.
struct RunParams {
    uint64_t seed;
    uint64_t event_base;
    uint64_t word_base;  // global index of the state's first 64-shot word
    uint64_t pad;
};

// A tile row holds the nq columns of a segment and kSegDummyCols zero
// columns (one per shared-memory bank group, for the pad lanes of gate
// groups), padded to an odd number of 16-byte cells so that the 8 words of
// one column fall on distinct bank groups.
constexpr int kSegDummyCols = 8;
__host__ __device__ inline int seg_row_cells(int nq) { return (nq + kSegDummyCols) | 1; }

// Row stride (in words) of a tile's record words [bw][stride]: a warp copies
// 32 / bw records of each of its bw words, so a stride of 32 / bw mod 16
// puts the 32 eight-byte stores on distinct bank pairs, two wavefronts.
__host__ __device__ inline int seg_rec_stride(int nrecsig, int bw) {
    if (bw < 2) return nrecsig;
    const int m = (32 / bw) % 16;
    return nrecsig + ((m - nrecsig % 16) % 16 + 16) % 16;
}

// A gate inside a fused segment (8 bytes).  a / b are LOCAL column indices
// (positions in the segment's touched-qubit list); code_rec holds the op code
// in its low 4 bits and, for the per-shot conditional gates, the record index
// above them.
struct SegGate {
    uint16_t a;
    uint16_t b;
    int32_t code_rec;
};

// A sign operation r ^= (fx & z_a) ^ (fz & x_a): the Pauli gates (constant
// masks, GateFunctors.hpp:303-307,323-327,372-376) and the X of a reset
// (mask = record outcome).
enum SignKind : int32_t { SIGN_X = 0, SIGN_Y = 1, SIGN_Z = 2, SIGN_REC_X = 3 };
struct SegSign {
    uint16_t a;
    uint16_t kind;
    int32_t rec;
};

// Layer L: gate runs [r0, r1) (all of its gates act on disjoint columns);
// afterwards sign ops [s0, s1) and the noise entries tagged with layer L.
struct SegLayer {
    int32_t r0, r1, s0, s1;
};

// A run of gates [g0, g1) of one code.  For H, S, CX and CZ the run is laid
// out in batches of 32 (one per warp instruction) whose columns fall evenly on
// the shared-memory banks, padded with gates on a zero dummy column; code -1
// marks a run of mixed / conditional gates.
struct SegRun {
    int32_t code, g0, g1, pad;
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

// Sampled channel outcome for one 64-shot word: X/Z components on local
// columns a and b (b = 0xFFFF for a one-qubit channel), applied after the
// gates of `layer`.
struct NoiseEntry {
    u64 fxa, fza, fxb, fzb;
    int32_t layer;
    uint16_t a;
    uint16_t b;
};

// Register-resident form of a segment.  Up to RC "resident" columns per lane
// (no gate of the segment joins two of them) stay in registers for the whole
// segment: the lane that owns one applies every gate on it, reading and
// writing only the partner column in shared memory.  ResOp is the owner's
// step for one (layer, slot): the gate code and the partner column.
enum ResCode : uint8_t { RS_NOP = 0, RS_H = 1, RS_S = 2, RS_CX_CTRL = 3, RS_CX_TGT = 4, RS_CZ = 5 };
struct ResOp {
    uint16_t other;  // partner tile column (two-qubit gates)
    uint8_t code;    // ResCode
    uint8_t pad;
};

// In the resident form sign ops and channel outcomes act after the last
// layer: a Pauli P applied after layer L flips the sign of exactly the rows
// that anticommute with it, and conjugating both by the remaining gates U
// keeps that relation, so the flip equals [row_end anticommutes with U P U^].
// prop_desc[i] = offset << 8 | length into prop_sup; prop_sup entries are
// column | x << 16 | z << 17 of the propagated Pauli (sign dropped).  Pauli i
// is component c (X_a, Z_a, X_b, Z_b) of channel slot s for i = 4s + c, and
// sign op k for i = 4 nslots + k.
constexpr uint32_t PROP_X = 1u << 16, PROP_Z = 1u << 17;

struct SegmentDev {
    const SegLayer *layers;
    int32_t nlayers;
    const SegRun *runs;
    int32_t nruns;
    const SegGate *gates;
    const SegSign *signs;
    const int32_t *cols;     // touched global qubits, nq entries
    int32_t nq;
    int32_t ngates;
    int32_t nsigns;
    // Reset-X sign ops carry a slot number (SegSign.rec); the record behind
    // slot i is recsig_rec[i].  Their outcome words are staged per tile.
    const int32_t *recsig_rec;
    int32_t nrecsig;
    const NoiseSlot *slots;
    int32_t nslots;
    const uint64_t *thr;     // threshold table
    NoiseEntry *entries;     // [w][cap]
    int32_t *entry_count;    // [w]
    int32_t cap;
    u64 *dense;              // [w][nslots][4] sampling scratch
    // resident form (res_slots > 0)
    int32_t word_vector;        // 1: word-vector form for one-row tiles
    int32_t res_slots;          // RC: register slots per lane
    const uint16_t *res_cols;   // [RC][32] tile column, 0xFFFF = empty
    const ResOp *res_ops;       // [nlayers][RC][32]
    const uint32_t *prop_desc;  // [4 nslots + nsigns]
    const uint32_t *prop_sup;
};

}  // namespace ps
