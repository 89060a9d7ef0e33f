// ps_frame.cu -- device side of shared-x/z runs (see ps_frame.h): the sign
// program over each shot-word's signs, and the broadcast of the final x / z
// bits to every shot.
#include <algorithm>

#include "ps_draw.cuh"
#include "ps_frame.h"
#include "ps_internal.h"
#include "ps_segment.cuh"

namespace ps {

namespace {

// One CTA of FW warps per shot-word: its W signs live in shared memory while
// it runs ops [op0, op1) in order.  Channel outcomes go one per thread over
// all warps (XORs commute; shared atomics where two outcomes flip one row),
// and so do the outputs of an F_LINEAR op; the other measurement ops (those
// the builder left out of its linear maps) run on warp 0 -- a window's
// measurements one per lane, the rows of other ops over the lanes -- with
// block barriers around every all-warp op.  When
// `stage` is set the launch's ops and the tab range [tab0, tab0 + ntab) of
// its measurement ops are first copied to shared memory, so the op stream
// runs on shared-memory latency; channel rows stay in global memory (a word
// uses few of them).  Record k of the circuit lives at rec + k*w (results)
// and rec + (nm + k)*w (determined flags).
constexpr int FW = 4;  // warps per shot-word

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem)
                 : "memory");
}

__global__ void __launch_bounds__(32 * FW, 4) frame_kernel(u64 *__restrict__ R, int64_t n, int64_t w,
                                                   const FrameOp *__restrict__ ops, uint32_t op0, uint32_t op1,
                                                   const uint32_t *__restrict__ tab, uint32_t tab0, uint32_t ntab16,
                                                   int stage, const uint32_t *__restrict__ slot_off,
                                                   const int32_t *__restrict__ rand_meas, uint32_t nrand,
                                                   const MeasOp *__restrict__ meas, u64 *__restrict__ rec,
                                                   int64_t nm, const NoiseEntry *__restrict__ entries,
                                                   int32_t *__restrict__ entry_count, int32_t cap, uint64_t seed,
                                                   const RunParams *__restrict__ rp, int from_zero,
                                                   int noise_first) {
    extern __shared__ u64 sR[];
    const int64_t W = 2 * n + 1;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t k = blockIdx.x;
    u64 *sout = sR + W + 1 + kWinRows;  // the launch's random outcomes, drawn up front
    uint32_t *stab = reinterpret_cast<uint32_t *>(((uintptr_t)(sout + nrand) + 15) & ~(uintptr_t)15);
    FrameOp *sops = reinterpret_cast<FrameOp *>(stab + 4 * ntab16);
    u64 *snew = reinterpret_cast<u64 *>(sops + (stage ? op1 - op0 : 0u));  // F_LINEAR's new rows
    // Signs, the tab range (16-byte chunks from the aligned tab0) and the ops
    // are copied asynchronously, all in flight at once, while the random
    // outcomes are drawn.
    if (from_zero) {
        for (int64_t i = tid; i < W; i += 32 * FW) sR[i] = 0ull;
    } else {
        for (int64_t i = tid; i < W; i += 32 * FW) cp_async8(&sR[i], R + i * w + k);
    }
    if (tid < 1 + (int)kWinRows) sR[W + tid] = 0ull;  // zero row (unused window reads), sinks (unused writes)
    if (stage) {
        for (uint32_t i = tid; i < ntab16; i += 32 * FW) cp_async16(stab + 4 * i, tab + tab0 + 4 * i);
        for (uint32_t i = tid; i < op1 - op0; i += 32 * FW) cp_async16(sops + i, ops + op0 + i);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    // A launch that starts with its segment's channel outcomes: each thread's
    // first outcome and its rows are fetched now, under the copies' latency.
    int pcnt = 0;
    NoiseEntry pen;
    pen.a = 0;
    uint32_t pv[kFrameChunk];
    if (noise_first) {
        pcnt = entry_count[k];
        if (tid < pcnt) pen = entries[k * (int64_t)cap + tid];
#pragma unroll
        for (uint32_t u = 0; u < kFrameChunk; ++u) pv[u] = u < pen.a ? tab[(uint32_t)pen.layer + u] : 0u;
    }
    const uint64_t event_base = rp->event_base, word_base = rp->word_base;
    for (uint32_t j = tid; j < nrand; j += 32 * FW)
        sout[j] = outcome_word(meas[rand_meas[j]], seed, event_base, k, word_base);
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    const uint32_t *T = stage ? stab : tab;  // measurement-op tab, indexed x - tb
    const uint32_t tb = stage ? tab0 : 0u;
    u64 last = 0ull;  // outcome of the latest measurement (its reset X)
    for (uint32_t oi = op0; oi < op1; ++oi) {
        const FrameOp o = stage ? sops[oi - op0] : ops[oi];
        const uint32_t kind = o.kind & 0xFFu;
        if (kind == F_NOISE) {
            __syncthreads();  // warp 0's measurement ops before
            auto apply = [&](const NoiseEntry &en, const uint32_t (&v)[kFrameChunk]) {
#pragma unroll
                for (uint32_t u = 0; u < kFrameChunk; ++u) {
                    if (v[u] == 0u) continue;  // a row entry is never 0 (sel != 0)
                    const uint32_t sel = v[u] >> 28;
                    u64 m = 0ull;
                    if (sel & 1u) m ^= en.fxa;
                    if (sel & 2u) m ^= en.fza;
                    if (sel & 4u) m ^= en.fxb;
                    if (sel & 8u) m ^= en.fzb;
                    atomicXor(&sR[v[u] & kFrameRowMask], m);
                }
            };
            const bool pre = noise_first && oi == op0;
            const int cnt = pre ? pcnt : entry_count[k];
            const NoiseEntry *ent = entries + k * (int64_t)cap;
            if (pre && tid < cnt) apply(pen, pv);
            for (int e = tid + (pre ? 32 * FW : 0); e < cnt; e += 32 * FW) {
                const NoiseEntry en = ent[e];  // layer: first row entry, a: row count (<= kFrameChunk)
                uint32_t v[kFrameChunk];
#pragma unroll
                for (uint32_t u = 0; u < kFrameChunk; ++u) v[u] = u < en.a ? tab[(uint32_t)en.layer + u] : 0u;
                apply(en, v);
            }
            __syncthreads();
            if (tid == 0) entry_count[k] = 0;  // consumed: the next segment's sampling appends from 0
        } else if (kind == F_LINEAR) {
            // every output from the signs as they were, then the new rows
            __syncthreads();  // warp 0's measurement ops before
            const uint32_t *L = T + (o.off - tb);
            const uint32_t nrec = L[0], nrow = L[1], nlast = L[2], nout = nrec + nrow + nlast;
            const uint32_t *dst = L + 4, *beg = dst + nout, *term = beg + nout + 1;
            for (uint32_t j = tid; j < nout; j += 32 * FW) {
                const uint32_t d = dst[j], t1 = beg[j + 1];
                u64 v = (d & kLinConst) ? ~0ull : 0ull;
#pragma unroll 4
                for (uint32_t t = beg[j]; t < t1; ++t) v ^= sR[term[t]];
                if (j < nrec) {
                    const int64_t m = (int64_t)(d & kLinIndex);
                    rec[m * w + k] = v;
                    rec[(nm + m) * w + k] = (d & kLinDet) ? ~0ull : 0ull;
                } else {
                    snew[j - nrec] = v;
                }
            }
            __syncthreads();
            for (uint32_t j = tid; j < nrow; j += 32 * FW) sR[dst[nrec + j] & kLinIndex] = snew[j];
            if (nlast) last = snew[nrow];
            __syncthreads();
        } else if (wid != 0) {
            continue;  // the measurement ops run on warp 0
        } else if (kind == F_WINDOW) {
            u64 acc = 0ull;
            uint32_t rs[kWinRows];
            if ((uint32_t)lane < o.len) {
                const uint32_t *rc = T + (o.off + kWinRec * lane - tb);
                const uint32_t m = rc[0], hdr = rc[1];
                uint32_t rd[kWinRows];
#pragma unroll
                for (uint32_t t = 0; t < kWinRows; ++t) {
                    rd[t] = rc[2 + t];
                    rs[t] = rc[2 + kWinRows + t];
                }
                acc = (hdr & 1u) ? ~0ull : 0ull;
#pragma unroll
                for (uint32_t t = 0; t < kWinRows; ++t) acc ^= sR[rd[t]];
                rec[(int64_t)m * w + k] = acc;
                rec[(nm + (int64_t)m) * w + k] = ~0ull;
                if ((uint32_t)lane == o.len - 1) sR[2 * n] = acc;
            }
            __syncwarp();
            if ((uint32_t)lane < o.len) {  // a lane's reset rows are distinct, and disjoint from other lanes' (sinks aside)
                u64 v[kWinRows];
#pragma unroll
                for (uint32_t t = 0; t < kWinRows; ++t) v[t] = sR[rs[t]];
#pragma unroll
                for (uint32_t t = 0; t < kWinRows; ++t) sR[rs[t]] = v[t] ^ acc;
            }
            last = __shfl_sync(0xffffffffu, acc, (int)o.len - 1);
            __syncwarp();
        } else if (kind == F_MEAS_DET) {
            u64 acc = 0ull;
            for (uint32_t t = o.off + lane; t < o.off + o.len; t += 32) acc ^= sR[T[t - tb]];
            acc = (u64)__reduce_xor_sync(0xffffffffu, (unsigned)(acc >> 32)) << 32 |
                  (u64)__reduce_xor_sync(0xffffffffu, (unsigned)acc);
            if (o.kind >> 8) acc = ~acc;
            if (lane == 0) {
                rec[(int64_t)o.arg * w + k] = acc;
                rec[(nm + (int64_t)o.arg) * w + k] = ~0ull;
                sR[2 * n] = acc;
            }
            last = acc;
            __syncwarp();
        } else if (kind == F_MEAS_RAND) {
            const u64 out = sout[o.kind >> 8];
            const uint32_t p = T[o.off - tb];
            const u64 rpv = sR[p + n];
            __syncwarp();
            if (lane == 0) {
                sR[p] = rpv;
                sR[p + n] = out;
                rec[(int64_t)o.arg * w + k] = out;
                rec[(nm + (int64_t)o.arg) * w + k] = 0ull;
            }
            // the multiplied rows exclude p and p+n (and are distinct): no barrier needed before them
            for (uint32_t t = o.off + 1 + lane; t < o.off + o.len; t += 32) {
                const uint32_t v = T[t - tb];
                sR[v & 0x7FFFFFFFu] ^= rpv ^ ((v >> 31) ? ~0ull : 0ull);
            }
            last = out;
            __syncwarp();
        } else {  // F_RESET_X, F_FLIP
            const u64 m = kind == F_RESET_X ? last : ~0ull;
            for (uint32_t t = o.off + lane; t < o.off + o.len; t += 32) sR[T[t - tb]] ^= m;
            __syncwarp();
        }
    }
    __syncthreads();
    for (int64_t i = tid; i < W; i += 32 * FW) R[i * w + k] = sR[i];
}

// x / z of every shot from the shared bits: one warp per (row, qubit), lanes
// over 16-byte word pairs.
__global__ void __launch_bounds__(256) broadcast_xz_kernel(XZBroadcast bc) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t rq = bc.rq0 + (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); rq < bc.rq1; rq += warps)
        broadcast_row_column(bc, rq, lane);
}

int g_frame_sms = 0;
int g_prio_greatest = 1;  // 1: not looked up yet (priorities are <= 0)
int g_prio_least = 1;

}  // namespace

size_t frame_smem_bytes(int64_t n) {  // rows, the zero row, kWinRows sink rows
    return (size_t)(2 * n + 2 + kWinRows) * sizeof(u64);
}

int launch_frame(cudaStream_t st, u64 *R, int64_t n, int64_t w, const FrameOp *ops, uint32_t op0, uint32_t op1,
                 const uint32_t *tab, uint32_t tab0, uint32_t tab1, const uint32_t *slot_off, const int32_t *rand_meas,
                 uint32_t nrand, const MeasOp *meas, u64 *rec, int64_t nm, const NoiseEntry *entries,
                 int32_t *entry_count, int32_t cap, uint64_t seed, const RunParams *rp, int from_zero,
                 int noise_first, uint32_t scratch) {
    // Staging keeps a CTA's shared memory small enough for two per SM.  The
    // staged tab range starts at tab0 rounded down to 16 bytes (tab holds
    // padding after its last word for the rounded-up end).  The F_LINEAR
    // scratch (new rows) comes last.
    const size_t base = ((frame_smem_bytes(n) + (size_t)nrand * sizeof(u64)) + 15) / 16 * 16;
    const uint32_t tab0a = tab0 & ~3u, tab1a = (tab1 + 3u) & ~3u;
    const size_t scr = (size_t)scratch * sizeof(u64);
    const size_t staged = base + (size_t)(tab1a - tab0a) * 4 + (size_t)(op1 - op0) * sizeof(FrameOp) + scr;
    const int stage = staged <= kFrameStageMax ? 1 : 0;
    const size_t smem = stage ? staged : base + scr;
    if (smem > kSegSmemMax) return E_ARG;
    const uint32_t ntab16 = stage ? (tab1a - tab0a) / 4 : 0u;
    if (smem > 48 * 1024) {
        const int rc = allow_max_smem((const void *)frame_kernel);
        if (rc != OK) return rc;
    }
    // The sign kernels are the plan's critical path: launched at the highest
    // priority, their CTAs go ahead of the side streams' queued sampling and
    // broadcast CTAs.
    if (g_prio_greatest == 1) {
        int least = 0, greatest = 0;
        PS_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        g_prio_greatest = greatest;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)w);
    cfg.blockDim = dim3(32 * FW);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = g_prio_greatest;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PS_CUDA(cudaLaunchKernelEx(&cfg, frame_kernel, R, n, w, ops, op0, op1, tab, tab0a, ntab16, stage, slot_off, rand_meas,
                               nrand, meas, rec, nm, entries, entry_count, cap, seed, rp, from_zero, noise_first));
    PS_CUDA(cudaGetLastError());
    return OK;
}

int launch_broadcast_xz(cudaStream_t st, const XZBroadcast &bc, bool yield) {
    if (bc.rq1 <= bc.rq0) return OK;
    if (g_frame_sms == 0) {
        int dev = 0;
        PS_CUDA(cudaGetDevice(&dev));
        PS_CUDA(cudaDeviceGetAttribute(&g_frame_sms, cudaDevAttrMultiProcessorCount, dev));
    }
    if (g_prio_least == 1) {
        int least = 0, greatest = 0;
        PS_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        g_prio_least = least;
    }
    // yield: one (row, qubit) pair per warp, so that CTAs retire within
    // microseconds and the kernels beside it (the sign program, launched at
    // the highest priority) get every SM slot that frees up; otherwise a
    // grid of 8 CTAs per SM walking the pairs.
    const int64_t pairs = bc.rq1 - bc.rq0;
    const int64_t blocks = yield ? (pairs + 7) / 8 : std::min<int64_t>((pairs + 7) / 8, (int64_t)g_frame_sms * 8);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = g_prio_least;
    cfg.attrs = attr;
    cfg.numAttrs = yield ? 1 : 0;
    PS_CUDA(cudaLaunchKernelEx(&cfg, broadcast_xz_kernel, bc));
    PS_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace ps
