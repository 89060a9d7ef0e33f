// ps_internal.h -- host-side structures shared by the library's translation
// units (not part of the public C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "ps_common.cuh"

namespace ps {

// One measurement record: bit-packed outcome and "determined" flag per shot,
// device resident (the reference keeps two int32 Views per record,
// CliffordState.hpp:32-58).  Host copies are filled lazily and dropped when
// the record is overwritten.
struct Record {
    int64_t qubit = -1;
    u64 *res = nullptr;  // device, w words
    u64 *det = nullptr;  // device, w words
    std::vector<u64> host_res, host_det;
    bool host_valid = false;
};

// Pool of fixed-size device blocks for records (one cudaMalloc per 64
// records instead of one per measurement).
struct RecordArena {
    std::vector<u64 *> chunks;
    size_t per_chunk = 64;
    size_t used_in_last = 0;
    size_t words = 0;  // words per record array
};

// Gate / op codes (same values as ps_op codes and the oracle's ORA_OP_*).
enum OpCode : int32_t {
    OP_H = 0, OP_S = 1, OP_X = 2, OP_Y = 3, OP_Z = 4, OP_CX = 5, OP_CZ = 6, OP_M = 7, OP_R = 8,
    OP_PAULI1 = 9, OP_PAULI2 = 10, OP_H_IF = 11, OP_S_IF = 12,
};

// One measurement for the measurement kernel.
struct MeasOp {
    int32_t q;
    int32_t reset;      // 1: X on shots with outcome 1 after measuring (ResetQubit)
    float bias;
    uint32_t event;     // Philox event index
    const u64 *forced;  // device packed bits (w words) or nullptr
    u64 *res;           // record words
    u64 *det;
};

} // namespace ps

struct ps_state {
    int64_t n = 0;      // qubits
    int64_t S = 0;      // shots (batch size)
    int64_t W = 0;      // 2n+1 rows
    int64_t w = 0;      // shot-words per column (padded to even)
    int64_t seed = 0;
    uint64_t events = 0;
    u64 *X = nullptr, *Z = nullptr, *R = nullptr;
    cudaStream_t stream = nullptr;
    // Device scratch for single-op calls.
    u64 *forced_buf = nullptr;   // w words
    u64 *mask_buf = nullptr;     // 4*w words (Pauli-channel masks)
    ps::MeasOp *meas_buf = nullptr;
    size_t meas_cap = 0;
    std::vector<ps::Record> recs;
    ps::RecordArena arena;
    int device = 0;
};

namespace ps {
// ps_state.cu
int state_alloc(ps_state *h, int64_t n, int64_t S, int64_t seed);
void state_free(ps_state *h);
int launch_init_zero(ps_state *h);
int record_new(ps_state *h, int64_t q, int64_t *id);
int record_fetch(ps_state *h, int64_t id);
int pack_from_host(ps_state *h, const int32_t *x, const int32_t *z, const int32_t *r);
int unpack_to_host(ps_state *h, int32_t *x, int32_t *z, int32_t *r);
int checksum(ps_state *h, int64_t s0, int64_t s1, int64_t *out);
int upload_forced(ps_state *h, const uint8_t *forced, const u64 **dev);

// ps_gates.cu
int launch_gate(ps_state *h, int32_t code, int64_t a, int64_t b, const u64 *flag);
int launch_pauli_channel(ps_state *h, int64_t a, int64_t b, const uint64_t *thresholds, int count);
// Sampling thresholds for a Pauli channel from float probabilities.
void channel_thresholds(const float *p, int count, uint64_t *thr);

// ps_measure.cu
int launch_measure(ps_state *h, const MeasOp *ops_host, int nops);
} // namespace ps
