// ps_internal.h -- host-side structures shared by the library's translation
// units (not part of the public C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

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
    std::vector<u64 *> blocks;  // contiguous blocks of compiled circuits
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
    int32_t *kstat;     // optional: {random branch taken, rows multiplied} of shot word 0
    int32_t pad;
};

// Sub-allocator over one device region reserved up front (the serving
// loop's HBM budget).  Bookkeeping is on the host only, so returning memory
// never synchronises the device; callers return a region only after the
// work that used it has finished.
struct DevPool {
    std::mutex mu;
    char *base = nullptr;
    size_t cap = 0, used = 0, peak = 0;
    std::map<size_t, size_t> free_;  // offset -> bytes, coalesced
    std::map<size_t, size_t> taken;  // offset -> bytes
    void reset(void *region, size_t bytes);
    bool alloc(void **p, size_t bytes);  // best fit, 256-byte granules
    void release(void *p);
};

} // namespace ps

struct ps_state {
    int64_t n = 0;      // qubits
    int64_t S = 0;      // shots (batch size)
    int64_t W = 0;      // 2n+1 rows
    int64_t w = 0;      // shot-words per column (padded to even)
    int64_t seed = 0;
    uint64_t events = 0;
    // Global index of the first 64-shot word: draws are keyed by global shot
    // words, so shot ranges split over several states (or GPUs) reproduce
    // the draws of one state holding all shots.
    int64_t word_base = 0;
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
    // True while the tableau is known to be a valid stabilizer tableau
    // (built from |0...0> by gates and measurements).  A tableau loaded from
    // the host may not be; compiled circuits then keep every reset's X
    // inside its measurement phase instead of deferring it.
    bool valid = false;
    // Device memory source: nullptr = cudaMalloc / cudaFree, else a pool.
    ps::DevPool *pool = nullptr;
    // Signs only: X and Z are not allocated.  Such a state runs only
    // compiled circuits whose shared-x/z plan runs from |0...0> and gives
    // only measurement records (the sampling jobs of the request loop).
    bool signs_only = false;
};

namespace ps {
// An NVTX range over a host scope (a run's enqueue, a launch kind, a served
// job): named ranges on the timeline of Nsight tools, a few nanoseconds
// when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    explicit NvtxRange(const std::string &name) { nvtxRangePushA(name.c_str()); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// ps_capi.cpp: records the entry point for error messages, clears the error.
void ps_enter(const char *method, int line);

// ps_state.cu
// Device memory of a state and of everything compiled for it.
int dev_alloc(ps_state *h, void **p, size_t bytes);
void dev_free(ps_state *h, void *p);
int state_alloc(ps_state *h, int64_t n, int64_t S, int64_t seed, DevPool *pool = nullptr, bool signs_only = false);
// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum, once per (kernel, device).  The limit is a process-wide property
// of the kernel, so it is only ever raised: launches from other host threads
// that asked for less are never invalidated between their check and launch.
int allow_max_smem(const void *kernel);
void state_free(ps_state *h);
int launch_init_zero(ps_state *h);
int launch_init_zero_on(cudaStream_t stream, ps_state *h);
int record_new(ps_state *h, int64_t q, int64_t *id);
// One contiguous device block for many records (results rows, then
// determined rows); the state owns it.
int record_block(ps_state *h, const std::vector<int64_t> &qubits, std::vector<int64_t> &ids, u64 **res_block,
                 u64 **det_block);
int record_fetch(ps_state *h, int64_t id);
int pack_from_host(ps_state *h, const int32_t *x, const int32_t *z, const int32_t *r);
int unpack_to_host(ps_state *h, int32_t *x, int32_t *z, int32_t *r);
int checksum(ps_state *h, int64_t s0, int64_t s1, int64_t *out);
int upload_forced(ps_state *h, const uint8_t *forced, const u64 **dev);

// ps_gates.cu
int launch_gate(ps_state *h, int32_t code, int64_t a, int64_t b, const u64 *flag);
int launch_pauli_channel(ps_state *h, int64_t a, int64_t b, const uint64_t *thresholds, int count);
// A Pauli channel's table (channel_word) from its float probabilities:
// count + 1 entries.
void channel_thresholds(const float *p, int count, uint64_t *thr);
// E_ARG unless every probability is finite and in [0, 1].  A table whose
// sum passes 1 is kept: its cumulative thresholds stop at 1, so the
// outcomes past that point are cut short in table order (the oracle and
// the committed fixtures define this).
int check_channel_probs(const float *p, int count);

// ps_measure.cu
struct RunParams;
int launch_measure(ps_state *h, const MeasOp *ops_host, int nops);
// words_per_cta: 1, 2 or 4 shot-words per CTA, 0 = automatic.
int launch_measure_list(cudaStream_t stream, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, const MeasOp *dev_ops,
                        int nops, uint64_t seed, uint64_t word_base, const RunParams *rp, int words_per_cta = 0);

// ps_segment.cu
struct SegmentDev;
size_t segment_smem_bytes(int nq, int rows, int bw);
// Shared memory of one segment launch: the tile plus the staged schedule.
size_t segment_launch_smem(int nlayers, int nruns, int ngates, int nsigns, int nq, int nrecsig, int rows, int bw,
                           int rc);
constexpr size_t kSegSmemMax = 227 * 1024;
// slot_tags: entries carry their slot index instead of their layer.
int launch_noise_sample(cudaStream_t stream, const SegmentDev &seg, int64_t w, const RunParams *rp,
                        int slot_tags = 0);
int launch_segment(cudaStream_t stream, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, const SegmentDev &seg,
                   int rows, int bw, int threads, const u64 *const *recs);

// ps_frame.cu (shared-x/z runs; the launches are declared in ps_frame_dev.h)
size_t frame_smem_bytes(int64_t n);
// Staging buffers of a sign program's ranges stay within this (beside the
// signs); ranges that need more read their ops from global memory.
constexpr size_t kFrameStageMax = 100 * 1024;

// ps_gates.cu (compiled-circuit form of the per-op kernels)
// The channel of a compiled plain run in one launch (sampling and sign
// flips); dev_surv: its table's survival products (channel_surv_table).
int launch_channel_apply(cudaStream_t st, ps_state *h, int64_t a, int64_t b, const uint64_t *dev_thr, int count,
                         const uint32_t *dev_surv, ChannelEst est, uint32_t event_off, const RunParams *rp);
int launch_channel_rp(cudaStream_t stream, ps_state *h, int64_t a, int64_t b, const uint64_t *dev_thr, int count,
                      uint32_t event_off, const RunParams *rp, u64 *dev_masks);
int launch_gate_on(cudaStream_t stream, ps_state *h, int32_t code, int64_t a, int64_t b, const u64 *flag);
} // namespace ps

struct ps_circuit;
namespace ps {
// ps_circuit.cpp: the pieces of a compiled circuit that batches drive.
int circuit_enqueue(ps_circuit *c, cudaStream_t st, bool reset);  // the plan, on any stream
RunParams circuit_begin_run(ps_circuit *c, bool reset);           // host bookkeeping of one run
RunParams *circuit_params_dev(ps_circuit *c);                     // device run parameters
RunParams circuit_current_params(const ps_circuit *c);             // the next run's, without taking them
ps_state *circuit_state(ps_circuit *c);
// ps_state.cu: device bytes state_alloc takes.
size_t state_bytes(int64_t n, int64_t S, bool signs_only = false);
}  // namespace ps

namespace ps {
// ps_gates.cu: Pauli channel on q whose scratch lives in a fixed device array.
int launch_pauli_channel_noalloc(ps_state *h, int64_t q, const uint64_t *thr3);
}  // namespace ps
