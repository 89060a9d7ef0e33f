// ps_frame.cu -- device side of shared-x/z runs (see ps_frame.h): the sign
// program of a whole run over each shot-word's signs in ONE launch, and the
// broadcast of the final x / z bits to every shot.  Both take a job table
// (ps_frame_dev.h): a single circuit is a table of one job, a batch of
// circuits is one table, so a batch run is these two launches too.
#include <algorithm>
#include <mutex>
#include <set>

#include "ps_draw.cuh"
#include "ps_frame_dev.h"

namespace ps {

namespace {

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(smem)), "l"(gmem)
                 : "memory");
}

// Bulk copies (TMA, no tensor map) into shared memory, completed on an
// mbarrier: one thread issues a copy of a whole contiguous block, every
// consumer polls the barrier's phase, at most kFrameWaitLimit times.
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t *bar, uint32_t bytes) {  // the one arrival, and its bytes
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t it = 0; it < kFrameWaitLimit; ++it) {
        uint32_t ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(ok)
                     : "r"(smem_u32(bar)), "r"(parity)
                     : "memory");
        if (ok) return true;
    }
    return false;
}

// The job of a CTA (or broadcast chunk) index: the last j with first[j] <= i.
__device__ __forceinline__ int job_of(const int64_t *__restrict__ first, int njobs, int64_t i) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(first + mid) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Bits 4 sub .. 4 sub + 3 of a random measurement's 64 outcomes of word k
// (Philox block `sub`, or the forced bits) -- outcome_bits split over 16
// lanes, so that one warp draws two measurements at once.
__device__ __forceinline__ u64 outcome_quarter(const MeasOp &op, int sub, uint64_t seed, uint64_t event_base,
                                               int64_t k, uint64_t word_base) {
    u64 bits = 0ull;
    if (op.forced) {
        const u64 fw = op.forced[k];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const int b = sub * 4 + l;
            const float u = ((fw >> b) & 1ull) ? 0.25f : 0.75f;
            if (u < op.bias) bits |= 1ull << b;
        }
    } else {
        const u32x4 u = draw_block(seed, event_base + op.event, word_base + (uint64_t)k, (uint32_t)sub, TAG_MEASURE);
#pragma unroll
        for (int l = 0; l < 4; ++l)
            if (unit_float(u.v[l]) < op.bias) bits |= 1ull << (sub * 4 + l);
    }
    return bits;
}

// One CTA of FW warps per shot-word k of a job runs the job's whole sign
// program on its W signs, held in shared memory from start (all zero: the
// run starts from |0...0>) to end.  Launch range by launch range:
//  1. its ops and measurement tab words are copied to shared memory with
//     cp.async (in flight during 2 and 3); the range's channel records were
//     fetched the same way during the range before;
//  2. the channel outcomes of its segment are drawn (the same draws as every
//     other form) and each outcome flips the signs of its slot's rows;
//  3. its random measurements' outcomes are drawn (they depend on no sign),
//     two per warp;
//  4. its ops run in order: F_LINEAR maps over all threads, other
//     measurement ops on warp 0 (a window's measurements one per lane, the
//     rows of other ops over the lanes).
// So the critical path reads shared memory only, but for one batched fetch
// of the hit channels' rows per range.  Records are written as they are
// produced; the signs go back to R at the end.  Record m of a job lives at
// rec + m*w (results) and rec + (nm + m)*w (determined flags).
// At most 85 registers a thread (3 CTAs of 8 warps, or 6 of 4, per SM's
// 64K): two sign CTAs then leave an SM room for the broadcast beside them.
template <int FW>
__global__ void __launch_bounds__(32 * FW, 24 / FW) frame_run_kernel(const FrameJobDev *__restrict__ jobs, int njobs,
                                                                     const int64_t *__restrict__ cta0) {
    extern __shared__ __align__(16) u64 sm[];
    constexpr int NT = 32 * FW;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int j = njobs > 1 ? job_of(cta0, njobs, (int64_t)blockIdx.x) : 0;
    const FrameJobDev &J = jobs[j];
    const int64_t n = J.n, w = J.w, W = 2 * n + 1, nm = J.nm;
    const int64_t k = (int64_t)blockIdx.x - cta0[j];
    const FrameSmem SL = frame_smem_layout(J);
    char *const sb8 = reinterpret_cast<char *>(sm);
    u64 *const sR = sm;  // signs, the zero row W, kWinRows sink rows
    u64 *const sout = reinterpret_cast<u64 *>(sb8 + SL.out);  // a range's random outcomes
    uint32_t *const stab = reinterpret_cast<uint32_t *>(sb8 + SL.tab);
    FrameOp *const sops = reinterpret_cast<FrameOp *>(sb8 + SL.ops);
    u64 *const snew = reinterpret_cast<u64 *>(sb8 + SL.nw);  // F_LINEAR's new rows
    FrameSlotDev *const sslot = reinterpret_cast<FrameSlotDev *>(sb8 + SL.slot);  // [2][max_slots rounded to 2]
    uint32_t *const ss64 = reinterpret_cast<uint32_t *>(sb8 + SL.s64);             // [2][max_slots rounded to 4]
    uint32_t *const srow = reinterpret_cast<uint32_t *>(sb8 + SL.row);             // the chunk's hit rows
    u64 *const shm = reinterpret_cast<u64 *>(sb8 + SL.hm);                         // the chunk's outcome masks (4 a hit)
    uint32_t *const shrow = reinterpret_cast<uint32_t *>(sb8 + SL.hrow);           // its first staged row (or ~0u)
    uint32_t *const shlen = reinterpret_cast<uint32_t *>(sb8 + SL.hlen);           // its staged row count
    uint32_t *const shpre = reinterpret_cast<uint32_t *>(sb8 + SL.hpre);           // prefix of the counts
    uint32_t *const swsum = reinterpret_cast<uint32_t *>(sb8 + SL.wsum);           // per-warp sums
    uint32_t *const shit = reinterpret_cast<uint32_t *>(sb8 + SL.hit);    // hit channels: count, then (channel, first draw)
    uint32_t *const srcnt = shit + 1;  // staged row words taken
    uint32_t *const shitl = shit + 2;
    uint64_t *const sbar = reinterpret_cast<uint64_t *>(sb8 + SL.bar);  // [0..1] channel records, [2] ops + tab
    const FrameOp *const gops = J.ops;
    const uint32_t *const gtab = J.tab;
    u64 *const rec = J.rec;
    const RunParams rp = *J.rp;
    // channel tables: staged once when small, else read where they are
    const FrameChanTab *ctab = J.ctab;
    const uint64_t *thr = J.thr;
    const uint32_t *surv = J.surv;
    if (J.stage_tabs) {
        FrameChanTab *c2 = reinterpret_cast<FrameChanTab *>(sb8 + SL.tabs);
        uint64_t *t2 = reinterpret_cast<uint64_t *>(c2 + J.n_ctab);
        uint32_t *s2 = reinterpret_cast<uint32_t *>(t2 + J.n_thr);
        for (uint32_t i = tid; i < J.n_ctab; i += NT) c2[i] = J.ctab[i];
        for (uint32_t i = tid; i < J.n_thr; i += NT) t2[i] = J.thr[i];
        for (uint32_t i = tid; i < J.n_surv; i += NT) s2[i] = J.surv[i];
        ctab = c2;
        thr = t2;
        surv = s2;
    }
    for (int64_t i = tid; i < W + 1 + (int64_t)kWinRows; i += NT) sR[i] = 0ull;
    // Bulk copies: the channel records and S_64 words of range li + 1 into
    // buffer (li + 1) & 1 (barrier sbar[(li + 1) & 1]) while range li runs,
    // and a range's ops and tab words at its start (sbar[2]); thread 0
    // issues them.  Barrier phases flip with every completed copy.
    if (tid == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(sbar + b);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    uint32_t pend = 0u;  // thread 0: the barriers with a copy in flight (bits 0..2)
    auto fetch_slots = [&](const FrameRangeDev &R, int buf) {  // thread 0; a range with channels
        const uint32_t rb = (((uint32_t)R.nslots + 1u) & ~1u) * (uint32_t)sizeof(FrameSlotDev),
                       sb = (((uint32_t)R.nslots + 3u) & ~3u) * 4u;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        pend |= 1u << buf;
        mbar_expect(sbar + buf, rb + sb);
        bulk_copy(sslot + (size_t)buf * ((J.max_slots + 1) & ~1u), J.slot + R.rec_base, rb, sbar + buf);
        bulk_copy(ss64 + (size_t)buf * ((J.max_slots + 3) & ~3u), J.slot_s64 + R.s64_base, sb, sbar + buf);
    };
    uint32_t sph[2] = {0u, 0u}, tph = 0u;  // the phases the next waits look for
    // Waits (every thread) for barrier b's copy.  False when a wait gave up
    // in any thread: the error word is set, the copies still in flight are
    // waited for (bounded), and the caller leaves the kernel.
    auto wait_bar = [&](int b) -> bool {
        uint32_t &ph = b < 2 ? sph[b] : tph;
        const bool ok = mbar_wait(sbar + b, ph);
        ph ^= 1u;
        if (__syncthreads_or(!ok) == 0) {
            pend &= ~(1u << b);
            return true;
        }
        if (tid == 0) {
            atomicOr(J.err, kFrameErrWait);
            for (int c = 0; c < 3; ++c)
                if ((pend >> c) & 1u) (void)mbar_wait(sbar + c, c == b ? (ph ^ 1u) : (c < 2 ? sph[c] : tph));
        }
        return false;
    };
    FrameRangeDev L = J.ranges[0];
    if (tid == 0 && L.nslots > 0) fetch_slots(L, 0);
    u64 last = 0ull;  // outcome of the latest measurement (its reset X)
    for (int li = 0; li < J.nranges; ++li) {
        const FrameRangeDev Ln = J.ranges[li + 1 < J.nranges ? li + 1 : li];  // in flight meanwhile
        if (tid == 0) {
            *shit = 0u;
            *srcnt = 0u;
            if (L.stage) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                pend |= 4u;
                mbar_expect(sbar + 2, L.ntab16 * 16u + (L.op1 - L.op0) * 16u);
                if (L.ntab16) bulk_copy(stab, gtab + L.tab0a, L.ntab16 * 16u, sbar + 2);
                if (L.op1 > L.op0) bulk_copy(sops, gops + L.op0, (L.op1 - L.op0) * 16u, sbar + 2);
            }
        }
        if (L.nslots > 0) {
            if (!wait_bar(li & 1)) return;
        } else {
            __syncthreads();
        }
        const FrameSlotDev *cs = sslot + (size_t)(li & 1) * ((J.max_slots + 1) & ~1u);
        const uint32_t *cs64 = ss64 + (size_t)(li & 1) * ((J.max_slots + 3) & ~3u);
        // 2. channel outcomes.  A first pass draws every channel's first
        //    number (a Philox block gives the first numbers of four channels;
        //    no shot of the word is hit unless it is at least S_64, 94 % of
        //    channels at p = 1e-3) with all lanes converged, and lists the
        //    hit channels with their first numbers.  Then a thread per hit
        //    samples its word (channel_word_est_hit: the same draws as every
        //    other form) and flips the signs of its slot's rows, prefetched
        //    meanwhile (32-bit shared atomics: XORs commute, and two slots
        //    may share a row).
        if (L.nslots > 0) {
            // every lane runs every iteration (the ballots below take the
            // full warp); channels past the end just report no hit.  With
            // consecutive events a warp takes 128 events at a time: lane t
            // draws the block of group t (events 4t .. 4t + 3), and in slice
            // q lane t takes event 32q + t, whose number it gets by shuffle,
            // so that the S_64 words are read contiguously.  Else one block
            // a channel.
            const uint64_t e0 = rp.event_base + (uint64_t)(L.ev0 >= 0 ? L.ev0 : 0);
            const uint64_t g0 = e0 >> 2;  // the first group
            const int64_t nunits = L.ev0 >= 0 ? (int64_t)(((e0 + (uint64_t)L.nslots - 1) >> 2) - g0 + 1)
                                              : (int64_t)L.nslots;
            auto append = [&](bool hit, uint32_t slot, uint32_t u) {  // warp-aggregated
                const unsigned b = __ballot_sync(0xffffffffu, hit);
                if (b == 0u) return;
                uint32_t base = 0u;
                if (lane == 0) base = atomicAdd(shit, (uint32_t)__popc(b));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (hit) {
                    const uint32_t at = base + __popc(b & ((1u << lane) - 1u));
                    shitl[2 * at] = slot;
                    shitl[2 * at + 1] = u;
                }
            };
            if (L.ev0 >= 0) {
                for (int64_t wb = 32 * (int64_t)wid; wb < nunits; wb += 32 * FW) {  // the warp's 32 groups
                    u32x4 blk{};
                    if (wb + lane < nunits)
                        blk = draw_block(rp.seed, g0 + (uint64_t)(wb + lane), rp.word_base + (uint64_t)k, 0u, TAG_NOISE_FIRST);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int src = 8 * q + (lane >> 2);
                        uint32_t x[4];
#pragma unroll
                        for (int c = 0; c < 4; ++c) x[c] = __shfl_sync(0xffffffffu, blk.v[c], src);
                        const uint32_t u = (lane & 3) == 0 ? x[0] : (lane & 3) == 1 ? x[1] : (lane & 3) == 2 ? x[2] : x[3];
                        const int64_t sl = (int64_t)(4 * (g0 + (uint64_t)wb)) + 32 * q + lane - (int64_t)e0;
                        const bool hit = sl >= 0 && sl < L.nslots && u >= cs64[sl];
                        append(hit, (uint32_t)sl, u);
                    }
                }
            } else {
                for (int64_t ub = 0; ub < nunits; ub += NT) {
                    const int64_t unit = ub + tid;
                    bool hit = false;
                    uint32_t u = 0u;
                    if (unit < nunits) {
                        u = channel_first_draw(rp.seed, rp.event_base + J.slot_event[L.slot_base + unit],
                                               rp.word_base + (uint64_t)k);
                        hit = u >= cs64[unit];
                    }
                    append(hit, (uint32_t)unit, u);
                }
            }
            __syncthreads();
            const uint32_t nhit = *shit;
            // The hits, kFrameHitChunk at a time.  A thread per hit (spread
            // over the warps: hit c0 + l on lane l / FW of warp l % FW)
            // stages the 16-byte-aligned cover of its slot's rows (16-byte
            // copies; tab holds padding after its end) and samples its word
            // meanwhile; then all threads apply the chunk's rows together,
            // row entry e on thread e % NT (the hit by binary search in the
            // prefix of the row counts), so that a long row list does not
            // hold the CTA back.
            for (uint32_t c0 = 0; c0 < nhit; c0 += kFrameHitChunk) {
                const uint32_t cend = min(nhit, c0 + kFrameHitChunk);
                if (tid == 0) *srcnt = 0u;
                __syncthreads();
                for (uint32_t l0 = 0; l0 < kFrameHitChunk; l0 += NT) {
                    const uint32_t l = l0 + (uint32_t)lane * FW + (uint32_t)wid, h = c0 + l;
                    if (h >= cend) continue;
                    const uint32_t s0 = shitl[2 * h];
                    const FrameSlotDev d = cs[s0];
                    const uint32_t len = d.lt >> 12, t0 = d.t0;
                    const uint32_t a0 = t0 & ~3u, span = ((t0 + len + 3u) & ~3u) - a0;
                    const uint32_t pos = atomicAdd(srcnt, span);
                    const bool staged = pos + span <= kFrameRowStage;
                    if (staged)
                        for (uint32_t c = 0; c < span; c += 4) cp_async16(srow + pos + c, gtab + a0 + c);
                    ChannelWord m{0ull, 0ull, 0ull, 0ull};
                    const uint32_t tb = d.lt & 0xFFFu;
                    if (tb != kFrameNoHit) {  // (a channel that never hits has S_64 = 2^32 - 1)
                        const FrameChanTab ct = ctab[tb];
                        const uint32_t ev = L.ev0 >= 0 ? (uint32_t)L.ev0 + s0 : J.slot_event[L.slot_base + s0];
                        m = channel_word_est_hit(rp.seed, rp.event_base + ev, rp.word_base + (uint64_t)k, shitl[2 * h + 1],
                                                 thr + ct.thr_off, ct.count, surv + ct.surv_off, ct.est);
                    }
                    shm[4 * (h - c0) + 0] = m.fxa;
                    shm[4 * (h - c0) + 1] = m.fza;
                    shm[4 * (h - c0) + 2] = m.fxb;
                    shm[4 * (h - c0) + 3] = m.fzb;
                    shrow[h - c0] = staged ? pos + (t0 - a0) : ~0u;
                    shlen[h - c0] = staged ? len : 0u;
                    if (!staged) {  // rows that do not fit: applied now, from global memory
                        for (uint32_t r = 0; r < len; ++r) {
                            const uint32_t v = __ldg(gtab + t0 + r), sel = v >> 28;
                            u64 f = 0ull;
                            if (sel & 1u) f ^= m.fxa;
                            if (sel & 2u) f ^= m.fza;
                            if (sel & 4u) f ^= m.fxb;
                            if (sel & 8u) f ^= m.fzb;
                            unsigned *rw = reinterpret_cast<unsigned *>(&sR[v & kFrameRowMask]);
                            if ((uint32_t)f) atomicXor(rw, (uint32_t)f);
                            if (f >> 32) atomicXor(rw + 1, (uint32_t)(f >> 32));
                        }
                    }
                }
                asm volatile("cp.async.commit_group;\n" ::: "memory");
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                __syncthreads();
                // exclusive prefix of the chunk's staged row counts: each
                // warp scans hits 32 w .. 32 w + 31 (every lane runs it)
                const uint32_t nh = cend - c0;
                uint32_t total = 0u;
                for (uint32_t b0 = 0; b0 < nh; b0 += NT) {
                    const uint32_t i = b0 + tid;
                    const uint32_t len = i < nh ? shlen[i] : 0u;
                    uint32_t x = len;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                        if (lane >= o) x += y;
                    }
                    if (lane == 31) swsum[wid] = x;
                    __syncthreads();
                    uint32_t woff = total, add = 0u;
#pragma unroll
                    for (int q = 0; q < FW; ++q) {
                        const uint32_t v = swsum[q];
                        woff += q < wid ? v : 0u;
                        add += v;
                    }
                    if (i < nh) shpre[i] = woff + x - len;
                    total += add;
                    __syncthreads();
                }
                for (uint32_t e = tid; e < total; e += NT) {
                    // the last hit with shpre <= e: it has staged rows (a hit
                    // without any shares its prefix with the next one, and
                    // the last one's prefix is the total)
                    uint32_t lo = 0u, hi = nh - 1u;
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1u) >> 1;
                        if (shpre[mid] <= e) lo = mid;
                        else hi = mid - 1u;
                    }
                    const uint32_t v = srow[shrow[lo] + (e - shpre[lo])], sel = v >> 28;
                    u64 f = 0ull;  // row | sel << 28: X on rows with z, Z on rows with x
                    if (sel & 1u) f ^= shm[4 * lo + 0];
                    if (sel & 2u) f ^= shm[4 * lo + 1];
                    if (sel & 4u) f ^= shm[4 * lo + 2];
                    if (sel & 8u) f ^= shm[4 * lo + 3];
                    unsigned *rw = reinterpret_cast<unsigned *>(&sR[v & kFrameRowMask]);
                    if ((uint32_t)f) atomicXor(rw, (uint32_t)f);
                    if (f >> 32) atomicXor(rw + 1, (uint32_t)(f >> 32));
                }
                __syncthreads();  // the chunk applied before the next one reuses the staging
            }
            __syncthreads();  // every hit applied before the ops
        }
        // the next range's channel records, into the buffer range li - 1 used
        if (tid == 0 && li + 1 < J.nranges && Ln.nslots > 0) fetch_slots(Ln, (li + 1) & 1);
        // 3. random outcomes: half-warps, one Philox block per lane
        for (uint32_t r0 = 2u * (uint32_t)wid; r0 < L.nrand; r0 += 2u * FW) {
            const uint32_t r = r0 + (uint32_t)(lane >> 4);
            u64 bits = 0ull;
            if (r < L.nrand)
                bits = outcome_quarter(J.meas[J.rand_meas[L.rand0 + r]], lane & 15, rp.seed, rp.event_base, k,
                                       rp.word_base);
#pragma unroll
            for (int off = 8; off > 0; off >>= 1) bits |= __shfl_xor_sync(0xffffffffu, bits, off);
            if ((lane & 15) == 0 && r < L.nrand) sout[r] = bits;
        }
        if (L.stage) {
            if (!wait_bar(2)) return;
        } else {
            __syncthreads();
        }
        // 4. the ops
        const uint32_t *T = L.stage ? stab : gtab;  // measurement-op tab, indexed x - tb
        const uint32_t tb = L.stage ? L.tab0a : 0u;
        for (uint32_t oi = L.op0; oi < L.op1; ++oi) {
            const FrameOp o = L.stage ? sops[oi - L.op0] : gops[oi];
            const uint32_t kind = o.kind & 0xFFu;
            if (kind == F_NOISE) continue;  // applied in 2 (always a range's first op)
            if (kind == F_LINEAR) {
                // every output from the signs as they were, then the new rows
                __syncthreads();  // warp 0's measurement ops before
                const uint32_t *Lm = T + (o.off - tb);
                const uint32_t nrec = Lm[0], nrow = Lm[1], nlast = Lm[2], nout = nrec + nrow + nlast;
                const uint32_t *dst = Lm + 4, *beg = dst + nout, *term = beg + nout + 1;
                for (uint32_t q = tid; q < nout; q += NT) {
                    const uint32_t d = dst[q], t1 = beg[q + 1];
                    u64 v = (d & kLinConst) ? ~0ull : 0ull;
#pragma unroll 4
                    for (uint32_t t = beg[q]; t < t1; ++t) v ^= sR[term[t]];
                    if (q < nrec) {
                        const int64_t m = (int64_t)(d & kLinIndex);
                        rec[m * w + k] = v;
                        rec[(nm + m) * w + k] = (d & kLinDet) ? ~0ull : 0ull;
                    } else {
                        snew[q - nrec] = v;
                    }
                }
                __syncthreads();
                for (uint32_t q = tid; q < nrow; q += NT) sR[dst[nrec + q] & kLinIndex] = snew[q];
                if (nlast) last = snew[nrow];
                __syncthreads();
            } else if (wid != 0) {
                continue;  // the other measurement ops run on warp 0
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
        __syncthreads();  // the range's ops done before the next range's staging and channel flips
        L = Ln;
    }
    for (int64_t i = tid; i < W; i += NT) J.R[i * w + k] = sR[i];
}

// x / z of every shot from the shared bits.  A warp takes one chunk: one
// (row, qubit) pair of a job whose rows are at least 32 words wide (lanes
// over 16-byte word pairs), or 32 / (w/2) pairs of a narrower one.  Chunks
// of a job are consecutive (chunk0).
__global__ void __launch_bounds__(256) broadcast_jobs_kernel(const BroadcastJobDev *__restrict__ jobs, int njobs,
                                                             const int64_t *__restrict__ chunk0, int64_t chunks) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < chunks; c += warps) {
        const int j = njobs > 1 ? job_of(chunk0, njobs, c) : 0;
        const BroadcastJobDev &B = jobs[j];
        const int64_t hw = B.w >> 1, pairs = (2 * B.n + 1) * B.n, local = c - chunk0[j];
        int64_t rq, kp0, step;
        if (hw >= 16) {
            rq = local;
            kp0 = lane;
            step = 32;
        } else {
            const int per = 32 / (int)hw;
            rq = local * per + lane / (int)hw;
            kp0 = lane % (int)hw;
            step = hw;
            if (lane >= per * (int)hw || rq >= pairs) continue;
        }
        const int64_t row = rq / B.n, q = rq - row * B.n;
        const u64 xb = (B.xz[(row * 2 + 0) * B.nw64 + (q >> 6)] >> (q & 63)) & 1ull;
        const u64 zb = (B.xz[(row * 2 + 1) * B.nw64 + (q >> 6)] >> (q & 63)) & 1ull;
        const ulonglong2 xv = make_ulonglong2(0ull - xb, 0ull - xb), zv = make_ulonglong2(0ull - zb, 0ull - zb);
        u64 *xo = B.X + rq * B.w, *zo = B.Z + rq * B.w;
        // streaming stores (evict first): the broadcast passes 1.65 GB through
        // L2 at d = 15 and must not evict the sign kernel's tables beside it
        for (int64_t kp = kp0; kp < hw; kp += step) {
            __stcs(reinterpret_cast<ulonglong2 *>(xo + 2 * kp), xv);
            __stcs(reinterpret_cast<ulonglong2 *>(zo + 2 * kp), zv);
        }
    }
}

int g_frame_sms = 0;
int g_prio_greatest = 1;  // 1: not looked up yet (priorities are <= 0)

// Both kernels of a run ask for the largest shared-memory carveout.  An SM
// changes its L1 / shared split only when it is idle, so a broadcast left to
// the default (no shared memory, an L1-heavy split) keeps the sign kernel's
// CTAs off every SM it occupies until it drains.
int same_carveout(const void *kernel) {
    static std::mutex mu;
    static std::set<std::pair<const void *, int>> done;
    int dev = 0;
    PS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({kernel, dev})) return OK;
    PS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared));
    done.insert({kernel, dev});
    return OK;
}

template <int FW>
int launch_frame_fw(cudaStream_t st, const FrameTable &t) {
    if (t.smem > 48 * 1024) {
        const int rc = allow_max_smem((const void *)frame_run_kernel<FW>);
        if (rc != OK) return rc;
    }
    {
        const int rc = same_carveout((const void *)frame_run_kernel<FW>);
        if (rc != OK) return rc;
    }
    // The sign kernel is the plan's critical path: launched at the highest
    // priority, its CTAs go ahead of the broadcast's queued CTAs.
    if (g_prio_greatest == 1) {
        int least = 0, greatest = 0;
        PS_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        g_prio_greatest = greatest;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)t.ctas);
    cfg.blockDim = dim3(32 * FW);
    cfg.dynamicSmemBytes = t.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = g_prio_greatest;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PS_CUDA(cudaLaunchKernelEx(&cfg, frame_run_kernel<FW>, t.jobs, (int)t.njobs, t.cta0));
    PS_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace

size_t frame_smem_bytes(int64_t n) {  // rows, the zero row, kWinRows sink rows
    return (size_t)(2 * n + 2 + kWinRows) * sizeof(u64);
}

int launch_frame_run(cudaStream_t st, const FrameTable &t, int warps) {
    if (t.njobs <= 0 || t.ctas <= 0) return OK;
    if (t.smem > kSegSmemMax) return fail(E_ARG, "sign program does not fit in shared memory");
    if (t.ctas > 0x7FFFFFFFll) return fail(E_ARG, "sign program: too many shot-words in one launch");
    switch (warps) {
    case 4: return launch_frame_fw<4>(st, t);
    case 0:
    case 8: return launch_frame_fw<8>(st, t);
    default: return fail(E_ARG, "sign kernel: 4 or 8 warps per CTA");
    }
}

int launch_broadcast_jobs(cudaStream_t st, const FrameTable &t, int ctas_per_sm) {
    if (t.njobs <= 0 || t.chunks <= 0) return OK;
    if (g_frame_sms == 0) {
        int dev = 0;
        PS_CUDA(cudaGetDevice(&dev));
        PS_CUDA(cudaDeviceGetAttribute(&g_frame_sms, cudaDevAttrMultiProcessorCount, dev));
    }
    {
        const int rc = same_carveout((const void *)broadcast_jobs_kernel);
        if (rc != OK) return rc;
    }
    const int per = ctas_per_sm > 0 ? ctas_per_sm : 2;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((t.chunks + 7) / 8, (int64_t)g_frame_sms * per));
    broadcast_jobs_kernel<<<(unsigned)blocks, 256, 0, st>>>(t.bjobs, t.njobs, t.chunk0, t.chunks);
    PS_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace ps
