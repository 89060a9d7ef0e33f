// ps_frame_dev.h -- device descriptors of shared-x/z runs (ps_frame.h): the
// job table of the one-launch sign-program kernel and of the x / z broadcast.
// A single circuit is a table of one job; a batch puts all of its jobs in one
// table, so each of the two kernels is one launch for the whole batch.
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
// kFrameTabStage bytes.  A range's hits are taken kFrameHitChunk at a time;
// their rows are staged in shared memory, up to kFrameRowStage words a chunk
// (a hit whose rows do not fit applies them alone, from global memory).
constexpr uint32_t kFrameTabStage = 4096;
constexpr uint32_t kFrameHitChunk = 256;
constexpr uint32_t kFrameRowStage = 2048;

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
    uint32_t pad[2];
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
};

// A sign CTA gives up on an asynchronous copy after this many polls of its
// barrier (each poll may suspend the thread for a while), sets the job's
// error word and leaves.
constexpr uint32_t kFrameWaitLimit = 1u << 22;
constexpr int32_t kFrameErrWait = 1;

// Shared-memory layout of the sign kernel for one job (byte offsets):
// signs (W rows, the zero row, kWinRows sink rows), random outcomes, staged
// tab words, staged ops, F_LINEAR's new rows, two buffers of channel
// records and two of their S_64 words (the range's, the next one's being
// fetched), the channel tables, the hit rows, a chunk of hits (outcome
// masks, first staged row, row count, prefix of the counts), per-warp sums,
// the hit list (count, staged row words, then channel and first draw of
// each hit), the barriers of the bulk copies (channel records: two, staged
// ops and tab words: one).
struct FrameSmem {
    size_t out, tab, ops, nw, slot, s64, tabs, row, hm, hrow, hlen, hpre, wsum, hit, bar, total;
};
__host__ __device__ inline size_t frame_align16(size_t x) { return (x + 15) & ~(size_t)15; }
__host__ __device__ inline FrameSmem frame_smem_layout(const FrameJobDev &j) {
    FrameSmem L;
    L.out = (size_t)(2 * j.n + 2 + kWinRows) * 8;
    L.tab = frame_align16(L.out + (size_t)j.max_rand * 8);
    L.ops = L.tab + (size_t)j.stage_u32 * 4;
    L.nw = L.ops + (size_t)j.max_ops * 16;
    L.slot = frame_align16(L.nw + (size_t)j.max_scratch * 8);
    L.s64 = frame_align16(L.slot + (size_t)2 * ((j.max_slots + 1) & ~1u) * sizeof(FrameSlotDev));
    L.tabs = frame_align16(L.s64 + (size_t)2 * ((j.max_slots + 3) & ~3u) * 4);
    L.row = frame_align16(L.tabs + (j.stage_tabs ? (size_t)j.n_ctab * sizeof(FrameChanTab) + (size_t)j.n_thr * 8 +
                                                       (size_t)j.n_surv * 4
                                                 : 0));
    L.hm = L.row + (size_t)kFrameRowStage * 4;
    L.hrow = L.hm + (size_t)kFrameHitChunk * 32;
    L.hlen = L.hrow + (size_t)kFrameHitChunk * 4;
    L.hpre = L.hlen + (size_t)kFrameHitChunk * 4;
    L.wsum = L.hpre + (size_t)kFrameHitChunk * 4;
    L.hit = L.wsum + 16 * 4;
    L.bar = frame_align16(L.hit + (size_t)(2 * j.max_slots + 2) * 4);
    L.total = L.bar + 32;
    return L;
}

// Shared memory the sign kernel needs for a job.
inline size_t frame_job_smem(const FrameJobDev &j) { return frame_smem_layout(j).total; }

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
// each job in the sign kernel, prefix sums of w) and chunk0[njobs + 1] (first
// broadcast chunk of each job, prefix sums of broadcast_chunks).
struct FrameTable {
    const FrameJobDev *jobs = nullptr;
    const BroadcastJobDev *bjobs = nullptr;
    const int64_t *cta0 = nullptr;
    const int64_t *chunk0 = nullptr;
    int32_t njobs = 0;
    int64_t ctas = 0, chunks = 0;  // totals
    size_t smem = 0;               // largest frame_job_smem of the table
};

// Sign-kernel warps per CTA the launch uses (4 or 8; 0 = 8).
int launch_frame_run(cudaStream_t st, const FrameTable &t, int warps);
// The x / z broadcast of every job; ctas_per_sm 0 = 2 (room for the sign
// kernel beside it on every SM).
int launch_broadcast_jobs(cudaStream_t st, const FrameTable &t, int ctas_per_sm);

}  // namespace ps
