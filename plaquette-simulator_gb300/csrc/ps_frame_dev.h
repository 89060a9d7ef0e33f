// ps_frame_dev.h -- device descriptors of shared-x/z runs (ps_frame.h): the
// job table of the three kernels of a run -- the channel noise of every
// range and shot-word, the one-launch sign program, the x / z broadcast.  A
// single circuit is a table of one job; a batch puts all of its jobs in one
// table, so each kernel is one launch for the whole batch.
#pragma once
#include "ps_frame.h"
#include "ps_internal.h"
#include "ps_segment.cuh"

namespace ps {

// A channel of a sign program, indexed like slot_off (slot_base + slot):
// its rows tab[t0, t0 + len) and its table, packed as lt = len << 12 |
// table; table kFrameNoHit marks a channel that never hits (total
// probability 0).  Its S_64 word (a first draw below it hits no shot of the
// word) and its event offset are kept in arrays of their own.
struct FrameSlotDev {
    uint32_t t0;
    uint32_t lt;
};
constexpr uint32_t kFrameNoHit = 4095;
constexpr uint32_t kFrameMaxTables = 4095;
constexpr uint32_t kFrameMaxSlotRows = (1u << 20) - 1;

// A distinct channel table: thresholds at thr + thr_off (count + 1 entries),
// survival products at surv + surv_off (channel_surv_table) and the factors
// of the sampler's estimates (channel_est_factors).
struct FrameChanTab {
    int32_t thr_off;
    int32_t count;
    uint32_t surv_off;
    uint32_t pad;
    ChannelEst est;
    uint32_t pad2[2];
};

// The channel tables are staged in shared memory when they take at most
// kFrameTabStage bytes.
constexpr uint32_t kFrameTabStage = 4096;

// One launch range of a sign program (FrameProgram::Launch): its segment's
// channel outcomes, drawn and applied first, then ops [op0, op1).
struct FrameRangeDev {
    int32_t nslots;          // the segment's channels (0: none)
    uint32_t slot_base;      // slot_off index of the segment's first slot
    uint32_t op0, op1;
    uint32_t tab0a, ntab16;  // staged tab words: 16-byte chunks from tab0a (stage = 1)
    uint32_t rand0, nrand;   // rand_meas[rand0, rand0 + nrand): the range's random measurements
    uint32_t stage;          // 1: ops and tab range staged in shared memory
    int32_t ev0;             // >= 0: the channels' events are ev0, ev0 + 1, ... (first draws by groups of four)
    uint32_t s64_base;       // slot_s64 index of the segment's first S_64 word (a multiple of 4)
    uint32_t rec_base;       // slot index of the segment's first channel record (even: 16-byte aligned)
    int32_t nv;              // >= 0: its noise vectors are block nv of the job's nvec
    uint32_t pad;
};

// One job: a sign program over the signs R of every shot-word of one state.
// The kernel runs one CTA per shot-word; CTA blocks of a job table are
// consecutive (FrameTable::cta0).
struct FrameJobDev {
    u64 *R;
    int64_t n, w;
    const FrameOp *ops;
    const uint32_t *tab;
    const FrameRangeDev *ranges;
    int32_t nranges;
    int32_t pad;
    const int32_t *rand_meas;
    const MeasOp *meas;
    u64 *rec;  // record block: results [nm][w], then determined [nm][w]
    int64_t nm;
    const uint64_t *thr;  // channel threshold tables
    const FrameSlotDev *slot;    // channel records, per range from rec_base
    const uint32_t *slot_s64;    // S_64 of every channel (0xFFFFFFFF for one that never hits), per range from s64_base
    const uint32_t *slot_event;  // event offset of every channel, like slot (ranges with ev0 < 0 read it)
    const FrameChanTab *ctab;
    const uint32_t *surv;
    const RunParams *rp;
    // sizes behind the shared-memory layout (FrameSmem): random outcomes,
    // staged tab words (a multiple of 4), staged ops, F_LINEAR's new rows,
    // channels of the largest segment, channel tables (ctab entries, thr
    // words, surv words; staged when stage_tabs = 1)
    uint32_t max_rand, stage_u32, max_ops, max_scratch, max_slots;
    uint32_t n_ctab, n_thr, n_surv, stage_tabs, pad2;
    int32_t *err;  // set to kFrameErrWait when a bounded wait gave up (the run's results are void)
    // Noise vectors: for the nnv ranges with channels (range index
    // nv_range[v]), the XOR that the range's channel outcomes make on the
    // signs of shot-word k: nvec[(v * w + k) * Wp + row], Wp = W rounded up
    // to even (16-byte rows).
    u64 *nvec;
    const int32_t *nv_range;
    int32_t nnv;
    int32_t pad3;
};
__host__ __device__ inline int64_t frame_wp(int64_t n) { return (2 * n + 2) & ~(int64_t)1; }

// A sign CTA gives up on an asynchronous copy after this many polls of its
// barrier (each poll may suspend the thread for a while), sets the job's
// error word and leaves.
constexpr uint32_t kFrameWaitLimit = 1u << 22;
constexpr int32_t kFrameErrWait = 1;

// Shared-memory layout of the sign kernel for one job (byte offsets):
// signs (W rows, the zero row, kWinRows sink rows), random outcomes, two
// buffers of staged tab words and ops (the range's, the next one's being
// fetched; buffer b's ops follow its tab words), F_LINEAR's new rows, two
// noise-vector buffers, the barriers of the bulk copies (noise vectors: two,
// staged tab words and ops: two).
struct FrameSmem {
    size_t out, tab, tabsz, nw, nv, bar, total;
};
__host__ __device__ inline size_t frame_align16(size_t x) { return (x + 15) & ~(size_t)15; }
__host__ __device__ inline FrameSmem frame_smem_layout(const FrameJobDev &j) {
    FrameSmem L;
    L.out = (size_t)(2 * j.n + 2 + kWinRows) * 8;
    L.tab = frame_align16(L.out + (size_t)j.max_rand * 8);
    L.tabsz = (size_t)j.stage_u32 * 4 + (size_t)j.max_ops * 16;  // one buffer
    L.nw = L.tab + 2 * L.tabsz;
    L.nv = frame_align16(L.nw + (size_t)j.max_scratch * 8);
    L.bar = L.nv + (j.nnv > 0 ? (size_t)2 * (size_t)frame_wp(j.n) * 8 : 0);
    L.total = L.bar + 32;
    return L;
}

// Shared memory the sign kernel needs for a job.
inline size_t frame_job_smem(const FrameJobDev &j) { return frame_smem_layout(j).total; }

// The noise kernel runs kNoiseWarps warps a CTA and takes the hits of its
// range kNoiseChunk (one per thread) at a time.
constexpr int kNoiseWarps = 4;
constexpr uint32_t kNoiseChunk = 32 * kNoiseWarps;
// The noise kernel asks for at least this much shared memory a CTA, which
// keeps it to six CTAs an SM.
constexpr size_t kNoiseSmemFloor = 36 * 1024;

// Shared-memory layout of the noise kernel for one job: the noise vector
// being summed (Wp words), a chunk of hits (outcome masks, first row entry,
// row count, prefix of the counts), per-warp sums, the channel tables when
// staged, the hit list (count, then channel and first draw of each hit).
struct NoiseSmem {
    size_t hm, ht0, hlen, hpre, wsum, tabs, hit, total;
};
__host__ __device__ inline NoiseSmem noise_smem_layout(const FrameJobDev &j) {
    NoiseSmem L;
    L.hm = (size_t)frame_wp(j.n) * 8;
    L.ht0 = L.hm + (size_t)kNoiseChunk * 32;
    L.hlen = L.ht0 + (size_t)kNoiseChunk * 4;
    L.hpre = L.hlen + (size_t)kNoiseChunk * 4;
    L.wsum = L.hpre + (size_t)kNoiseChunk * 4;
    L.tabs = L.wsum + 16 * 4;
    L.hit = frame_align16(L.tabs + (j.stage_tabs ? (size_t)j.n_ctab * sizeof(FrameChanTab) + (size_t)j.n_thr * 8 +
                                                       (size_t)j.n_surv * 4
                                                 : 0));
    L.total = L.hit + (size_t)(2 * j.max_slots + 2) * 4;
    return L;
}
inline size_t noise_job_smem(const FrameJobDev &j) { return noise_smem_layout(j).total; }

// One job of the x / z broadcast: X and Z of every (row, qubit) pair and
// shot-word := the shared bits xz ([W][2][nw64]).
struct BroadcastJobDev {
    u64 *X, *Z;
    const uint64_t *xz;
    int64_t n, w, nw64;
};

// Broadcast warp chunks of a job: one (row, qubit) pair per chunk when a
// row is at least 32 words wide, else 32 / (w/2) pairs per chunk.
inline int64_t broadcast_chunks(int64_t n, int64_t w) {
    const int64_t pairs = (2 * n + 1) * n, hw = w / 2;
    if (hw >= 16) return pairs;
    const int64_t per = 32 / (hw > 0 ? hw : 1);
    return (pairs + per - 1) / per;
}

// A table of jobs on the device: jobs[njobs], cta0[njobs + 1] (first CTA of
// each job in the sign kernel, prefix sums of w), ncta0[njobs + 1] (first CTA
// of each job in the noise kernel, prefix sums of nnv * w) and chunk0[njobs +
// 1] (first broadcast chunk of each job, prefix sums of broadcast_chunks).
struct FrameTable {
    const FrameJobDev *jobs = nullptr;
    const BroadcastJobDev *bjobs = nullptr;
    const int64_t *cta0 = nullptr;
    const int64_t *ncta0 = nullptr;
    const int64_t *chunk0 = nullptr;
    int32_t njobs = 0;
    int64_t ctas = 0, nctas = 0, chunks = 0;  // totals
    size_t smem = 0;                          // largest frame_job_smem of the table
    size_t nsmem = 0;                         // largest noise_job_smem of the table
    // two zeroed words (the broadcast's chunk counter and finished-CTA
    // count; zero again after every launch); null: a static chunk split
    unsigned long long *bctr = nullptr;
};
// Broadcast chunks a warp takes from the counter at a time.
constexpr int64_t kBcastBatch = 8;

// The noise vectors of every job (nothing when no job has channels).
int launch_noise_vectors(cudaStream_t st, const FrameTable &t);
// Sign-kernel warps per CTA the launch uses (4 or 8; 0 = 8).
int launch_frame_run(cudaStream_t st, const FrameTable &t, int warps);
// ps_circuit.cpp: a run of every job of a table from |0...0> (run
// parameters on the device already): the broadcast on `side` (forked from
// st with `fork`, joined back with `join`) beside the noise vectors and the
// sign program on st; side = nullptr runs the three in order on st.
int frame_table_enqueue(const FrameTable &t, cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join,
                        int warps, int bctas);
// The fastest (sign-kernel warps, broadcast CTAs per SM) for a table, by
// timing each candidate's run; the tableaux and records are left holding
// the timed runs' data.
int frame_table_tune(const FrameTable &t, cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join,
                     int *warps, int *bctas, double *best_ms);
// A compiled circuit's entries for a batch's table (false: the circuit does
// not run the shared-x/z plan).
bool circuit_frame_job(const ps_circuit *c, FrameJobDev *job, BroadcastJobDev *bjob);

// The x / z broadcast of every job; ctas_per_sm 0 = 1 (eight warps an SM
// write at close to the copy rate and leave the noise and sign kernels
// most of each SM and of the memory system).
int launch_broadcast_jobs(cudaStream_t st, const FrameTable &t, int ctas_per_sm);

}  // namespace ps
