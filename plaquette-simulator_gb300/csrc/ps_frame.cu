// ps_frame.cu -- device side of shared-x/z runs (see ps_frame.h): three
// kernels a run, each one launch for a whole job table (ps_frame_dev.h):
//  - noise_vec_kernel: for every range with channels and every shot-word,
//    the XOR that the range's channel outcomes make on the signs (one CTA
//    each, independent of the signs, so all of them at once);
//  - frame_run_kernel: the sign program of a whole run over each shot-word's
//    signs, held in shared memory from start to end;
//  - broadcast_jobs_kernel: the final x / z bits written to every shot,
//    beside the other two.
#include <algorithm>
#include <mutex>
#include <set>

#include "ps_draw.cuh"
#include "ps_frame_dev.h"

namespace ps {

namespace {

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

// One CTA of NW warps per (range with channels, shot-word) of a job: the
// XOR its channel outcomes make on the signs of the word's 64 shots.  A
// first pass draws every channel's first number (a Philox block gives the
// first numbers of four consecutive channel events: lane t draws the block
// of group t, and in slice q lane t takes event 32q + t, whose number it
// gets by shuffle, so that the S_64 words are read contiguously; no shot of
// the word is hit unless the number is at least S_64, 94 % of channels at
// p = 1e-3) and lists the hit channels with their first numbers.  Then a
// thread per hit samples its word (channel_word_est_hit: the same draws as
// every other form) and flips its slot's rows in the sum (32-bit shared
// atomics: XORs commute, and two slots may share a row).
template <int NW>
__global__ void __launch_bounds__(32 * NW) noise_vec_kernel(const FrameJobDev *__restrict__ jobs, int njobs,
                                                            const int64_t *__restrict__ ncta0) {
    extern __shared__ __align__(16) u64 sm[];
    constexpr int NT = 32 * NW;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int j = njobs > 1 ? job_of(ncta0, njobs, (int64_t)blockIdx.x) : 0;
    const FrameJobDev &J = jobs[j];
    const int64_t w = J.w, Wp = frame_wp(J.n);
    const int64_t local = (int64_t)blockIdx.x - ncta0[j];
    const int64_t v = local / w, k = local - v * w;
    const FrameRangeDev L = J.ranges[J.nv_range[v]];
    const NoiseSmem SL = noise_smem_layout(J);
    char *const sb8 = reinterpret_cast<char *>(sm);
    u64 *const acc = sm;
    uint32_t *const shit = reinterpret_cast<uint32_t *>(sb8 + SL.hit);  // hit channels: count, then (channel, first draw)
    uint32_t *const shitl = shit + 2;
    u64 *const shm = reinterpret_cast<u64 *>(sb8 + SL.hm);               // the chunk's outcome masks (4 a hit)
    uint32_t *const sht0 = reinterpret_cast<uint32_t *>(sb8 + SL.ht0);   // first row entry of each
    uint32_t *const shlen = reinterpret_cast<uint32_t *>(sb8 + SL.hlen); // its row count
    uint32_t *const shpre = reinterpret_cast<uint32_t *>(sb8 + SL.hpre); // prefix of the counts
    uint32_t *const swsum = reinterpret_cast<uint32_t *>(sb8 + SL.wsum); // per-warp sums
    const uint32_t *const gtab = J.tab;
    const RunParams rp = *J.rp;
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
    for (int64_t i = tid; i < Wp; i += NT) acc[i] = 0ull;
    if (tid == 0) *shit = 0u;
    __syncthreads();
    const uint32_t *const s64 = J.slot_s64 + L.s64_base;
    const FrameSlotDev *const rec = J.slot + L.rec_base;
    auto append = [&](bool hit, uint32_t slot, uint32_t u) {  // warp-aggregated; every lane calls it
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
        const uint64_t e0 = rp.event_base + (uint64_t)L.ev0, g0 = e0 >> 2;
        const int64_t ngroups = (int64_t)(((e0 + (uint64_t)L.nslots - 1) >> 2) - g0 + 1);
        for (int64_t wb = 32 * (int64_t)wid; wb < ngroups; wb += 32 * NW) {  // the warp's 32 groups
            u32x4 blk{};
            if (wb + lane < ngroups)
                blk = draw_block(rp.seed, g0 + (uint64_t)(wb + lane), rp.word_base + (uint64_t)k, 0u, TAG_NOISE_FIRST);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int src = 8 * q + (lane >> 2);
                uint32_t x[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) x[c] = __shfl_sync(0xffffffffu, blk.v[c], src);
                const uint32_t u = (lane & 3) == 0 ? x[0] : (lane & 3) == 1 ? x[1] : (lane & 3) == 2 ? x[2] : x[3];
                const int64_t sl = (int64_t)(4 * (g0 + (uint64_t)wb)) + 32 * q + lane - (int64_t)e0;
                const bool hit = sl >= 0 && sl < L.nslots && u >= __ldg(s64 + sl);
                append(hit, (uint32_t)sl, u);
            }
        }
    } else {
        for (int64_t ub = 0; ub < L.nslots; ub += NT) {
            const int64_t unit = ub + tid;
            bool hit = false;
            uint32_t u = 0u;
            if (unit < L.nslots) {
                u = channel_first_draw(rp.seed, rp.event_base + J.slot_event[L.slot_base + unit], rp.word_base + (uint64_t)k);
                hit = u >= __ldg(s64 + unit);
            }
            append(hit, (uint32_t)unit, u);
        }
    }
    __syncthreads();
    // The hits, NT at a time: a thread per hit (spread over the warps: hit
    // c0 + l on lane l / NW of warp l % NW) samples its word, then all
    // threads apply the chunk's rows together, row entry e on thread e % NT
    // (its hit by binary search in the prefix of the row counts), so that a
    // long row list does not hold its warp back.
    const uint32_t nhit = *shit;
    for (uint32_t c0 = 0; c0 < nhit; c0 += NT) {
        const uint32_t l = (uint32_t)lane * NW + (uint32_t)wid, h = c0 + l;
        uint32_t len = 0u;
        if (h < nhit) {
            const uint32_t s0 = shitl[2 * h];
            const FrameSlotDev d = rec[s0];
            const uint32_t tb = d.lt & 0xFFFu;
            ChannelWord m{0ull, 0ull, 0ull, 0ull};
            if (tb != kFrameNoHit) {  // (a channel that never hits has S_64 = 2^32 - 1)
                const FrameChanTab ct = ctab[tb];
                const uint32_t ev = L.ev0 >= 0 ? (uint32_t)L.ev0 + s0 : J.slot_event[L.slot_base + s0];
                m = channel_word_est_hit(rp.seed, rp.event_base + ev, rp.word_base + (uint64_t)k, shitl[2 * h + 1],
                                         thr + ct.thr_off, ct.count, surv + ct.surv_off, ct.est);
                len = d.lt >> 12;
            }
            shm[4 * l + 0] = m.fxa;
            shm[4 * l + 1] = m.fza;
            shm[4 * l + 2] = m.fxb;
            shm[4 * l + 3] = m.fzb;
            sht0[l] = d.t0;
        }
        shlen[l] = len;
        __syncthreads();
        // exclusive prefix of the row counts, in chunk order (thread tid
        // takes entry tid here)
        const uint32_t mine = shlen[tid];
        uint32_t x = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) swsum[wid] = x;
        __syncthreads();
        uint32_t woff = 0u, total = 0u;
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const uint32_t vq = swsum[q];
            woff += q < wid ? vq : 0u;
            total += vq;
        }
        shpre[tid] = woff + x - mine;
        __syncthreads();
        for (uint32_t e = tid; e < total; e += NT) {
            // the last hit with shpre <= e: it has rows (one without any
            // shares its prefix with the next, and the last one's prefix is
            // the total)
            uint32_t lo = 0u, hi = NT - 1u;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1u) >> 1;
                if (shpre[mid] <= e) lo = mid;
                else hi = mid - 1u;
            }
            const uint32_t vr = __ldg(gtab + sht0[lo] + (e - shpre[lo])), sel = vr >> 28;
            u64 f = 0ull;  // row | sel << 28: X on rows with z, Z on rows with x
            if (sel & 1u) f ^= shm[4 * lo + 0];
            if (sel & 2u) f ^= shm[4 * lo + 1];
            if (sel & 4u) f ^= shm[4 * lo + 2];
            if (sel & 8u) f ^= shm[4 * lo + 3];
            unsigned *rw = reinterpret_cast<unsigned *>(&acc[vr & kFrameRowMask]);
            if ((uint32_t)f) atomicXor(rw, (uint32_t)f);
            if (f >> 32) atomicXor(rw + 1, (uint32_t)(f >> 32));
        }
        __syncthreads();  // the chunk applied before the next one reuses its arrays
    }
    __syncthreads();
    u64 *const out = J.nvec + ((int64_t)v * w + k) * Wp;
    for (int64_t i = tid; i < Wp; i += NT) out[i] = acc[i];
}

// One CTA of FW warps per shot-word k of a job runs the job's whole sign
// program on its W signs, held in shared memory from start (all zero: the
// run starts from |0...0>) to end.  Launch range by launch range:
//  1. its ops and measurement tab words come to shared memory by a bulk
//     copy (in flight during 2 and 3), and so does the noise vector of the
//     next range with channels;
//  2. its own noise vector (fetched during the range before) is XORed into
//     the signs;
//  3. its random measurements' outcomes are drawn (they depend on no sign),
//     two per warp;
//  4. its ops run in order: F_LINEAR maps over all threads, other
//     measurement ops on warp 0 (a window's measurements one per lane, the
//     rows of other ops over the lanes).
// Records are written as they are produced; the signs go back to R at the
// end.  Record m of a job lives at rec + m*w (results) and rec + (nm + m)*w
// (determined flags).  At most 85 registers a thread (3 CTAs of 8 warps,
// or 6 of 4, per SM's 64K): two sign CTAs then leave an SM room for the
// broadcast beside them.
template <int FW>
__global__ void __launch_bounds__(32 * FW, 24 / FW) frame_run_kernel(const FrameJobDev *__restrict__ jobs, int njobs,
                                                                     const int64_t *__restrict__ cta0) {
    extern __shared__ __align__(16) u64 sm[];
    constexpr int NT = 32 * FW;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int j = njobs > 1 ? job_of(cta0, njobs, (int64_t)blockIdx.x) : 0;
    const FrameJobDev &J = jobs[j];
    const int64_t n = J.n, w = J.w, W = 2 * n + 1, nm = J.nm, wp = frame_wp(n);
    const int64_t k = (int64_t)blockIdx.x - cta0[j];
    const FrameSmem SL = frame_smem_layout(J);
    char *const sb8 = reinterpret_cast<char *>(sm);
    u64 *const sR = sm;  // signs, the zero row W, kWinRows sink rows
    u64 *const sout = reinterpret_cast<u64 *>(sb8 + SL.out);  // a range's random outcomes
    u64 *const snew = reinterpret_cast<u64 *>(sb8 + SL.nw);  // F_LINEAR's new rows
    u64 *const snv = reinterpret_cast<u64 *>(sb8 + SL.nv);   // [2][wp] noise vectors
    uint64_t *const sbar = reinterpret_cast<uint64_t *>(sb8 + SL.bar);  // [0..1] noise vectors, [2..3] tab + ops
    // staging buffer b: tab words, then ops
    auto stab_of = [&](int b) { return reinterpret_cast<uint32_t *>(sb8 + SL.tab + (size_t)b * SL.tabsz); };
    auto sops_of = [&](int b) {
        return reinterpret_cast<FrameOp *>(sb8 + SL.tab + (size_t)b * SL.tabsz + (size_t)J.stage_u32 * 4);
    };
    const FrameOp *const gops = J.ops;
    const uint32_t *const gtab = J.tab;
    u64 *const rec = J.rec;
    const RunParams rp = *J.rp;
    for (int64_t i = tid; i < W + 1 + (int64_t)kWinRows; i += NT) sR[i] = 0ull;
    // Bulk copies, issued by thread 0 while range li runs: the noise vector
    // of range li + 1 (when it has channels) into buffer (li + 1) & 1
    // (barrier sbar[(li + 1) & 1]), and its staged tab words and ops into
    // buffer (li + 1) & 1 (barrier sbar[2 + ((li + 1) & 1)]).  Barrier
    // phases flip with every completed copy.
    if (tid == 0) {
        for (int b = 0; b < 4; ++b) mbar_init(sbar + b);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    uint32_t pend = 0u;  // thread 0: the barriers with a copy in flight (bits 0..3)
    auto fetch_nv = [&](const FrameRangeDev &R, int buf) {  // thread 0; a range with channels
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        pend |= 1u << buf;
        mbar_expect(sbar + buf, (uint32_t)(wp * 8));
        bulk_copy(snv + (int64_t)buf * wp, J.nvec + ((int64_t)R.nv * w + k) * wp, (uint32_t)(wp * 8), sbar + buf);
    };
    auto fetch_tab = [&](const FrameRangeDev &R, int buf) {  // thread 0; a staged range
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        pend |= 4u << buf;
        mbar_expect(sbar + 2 + buf, R.ntab16 * 16u + (R.op1 - R.op0) * 16u);
        if (R.ntab16) bulk_copy(stab_of(buf), gtab + R.tab0a, R.ntab16 * 16u, sbar + 2 + buf);
        if (R.op1 > R.op0) bulk_copy(sops_of(buf), gops + R.op0, (R.op1 - R.op0) * 16u, sbar + 2 + buf);
    };
    uint32_t ph[4] = {0u, 0u, 0u, 0u};  // the phases the next waits look for
    // Waits (every thread) for barrier b's copy.  False when a wait gave up
    // in any thread: the error word is set, the copies still in flight are
    // waited for (bounded), and the caller leaves the kernel.
    auto wait_bar = [&](int b) -> bool {
        const bool ok = mbar_wait(sbar + b, ph[b]);
        ph[b] ^= 1u;
        if (__syncthreads_or(!ok) == 0) {
            pend &= ~(1u << b);
            return true;
        }
        if (tid == 0) {
            atomicOr(J.err, kFrameErrWait);
            for (int c = 0; c < 4; ++c)
                if ((pend >> c) & 1u) (void)mbar_wait(sbar + c, c == b ? (ph[c] ^ 1u) : ph[c]);
        }
        return false;
    };
    FrameRangeDev L = J.ranges[0];
    if (tid == 0 && L.nv >= 0) fetch_nv(L, 0);
    if (tid == 0 && L.stage) fetch_tab(L, 0);
    u64 last = 0ull;  // outcome of the latest measurement (its reset X)
    for (int li = 0; li < J.nranges; ++li) {
        const FrameRangeDev Ln = J.ranges[li + 1 < J.nranges ? li + 1 : li];  // in flight meanwhile
        // the next range's tab words and ops, into the buffer the range before used
        if (tid == 0 && li + 1 < J.nranges && Ln.stage) fetch_tab(Ln, (li + 1) & 1);
        // 2. the range's channel outcomes (its first op, F_NOISE)
        if (L.nv >= 0) {
            if (!wait_bar(li & 1)) return;
            const u64 *nv = snv + (int64_t)(li & 1) * wp;
            for (int64_t i = tid; i < W; i += NT) sR[i] ^= nv[i];
        }
        // the next range's noise vector, into the buffer the range before used
        if (tid == 0 && li + 1 < J.nranges && Ln.nv >= 0) fetch_nv(Ln, (li + 1) & 1);
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
            if (!wait_bar(2 + (li & 1))) return;
        } else {
            __syncthreads();
        }
        const uint32_t *const stab = stab_of(li & 1);
        const FrameOp *const sops = sops_of(li & 1);
        // 4. the ops
        const uint32_t *T = L.stage ? stab : gtab;  // measurement-op tab, indexed x - tb
        const uint32_t tb = L.stage ? L.tab0a : 0u;
        for (uint32_t oi = L.op0; oi < L.op1; ++oi) {
            const FrameOp o = L.stage ? sops[oi - L.op0] : gops[oi];
            const uint32_t kind = o.kind & 0xFFu;
            if (kind == F_NOISE) continue;  // applied in 2
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
        __syncthreads();  // the range's ops done before the next range's staging and noise
        L = Ln;
    }
    for (int64_t i = tid; i < W; i += NT) J.R[i * w + k] = sR[i];
}

// One (row, qubit) chunk c of job B (local index `local`) by one warp: a
// whole row of shot-words when the row is at least 32 words wide, else
// 32 / (w/2) pairs side by side.
__device__ __forceinline__ void broadcast_chunk(const BroadcastJobDev &B, int64_t local, int lane) {
    const int64_t hw = B.w >> 1, pairs = (2 * B.n + 1) * B.n;
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
        if (lane >= per * (int)hw || rq >= pairs) return;
    }
    const int64_t row = rq / B.n, q = rq - row * B.n;
    const u64 xb = (B.xz[(row * 2 + 0) * B.nw64 + (q >> 6)] >> (q & 63)) & 1ull;
    const u64 zb = (B.xz[(row * 2 + 1) * B.nw64 + (q >> 6)] >> (q & 63)) & 1ull;
    const ulonglong2 xv = make_ulonglong2(0ull - xb, 0ull - xb), zv = make_ulonglong2(0ull - zb, 0ull - zb);
    u64 *xo = B.X + rq * B.w, *zo = B.Z + rq * B.w;
    for (int64_t kp = kp0; kp < hw; kp += step) {
        __stcs(reinterpret_cast<ulonglong2 *>(xo + 2 * kp), xv);
        __stcs(reinterpret_cast<ulonglong2 *>(zo + 2 * kp), zv);
    }
}

// The x / z broadcast of every job of a table: X and Z of each (row, qubit)
// pair and shot-word := the shared bits.  Stores are streaming (evict
// first): the broadcast passes 1.65 GB through L2 at d = 15 and must not
// evict the tables of the kernels beside it.  At most 32 registers a
// thread: two broadcast CTAs (16K registers) fit on an SM beside six noise
// CTAs (48K) or two sign CTAs (40K).
//
// With a counter (ctr), warps take kBcastBatch chunks at a time from it, so
// CTAs that reach their SMs late (beside the other kernels of the run) take
// less of the work; the last CTA to finish puts the counter back to zero
// for the next launch.  Without one, warp i takes chunks i, i + warps, ...
// ONE: a table of one job (no job lookup).
template <bool ONE>
__global__ void __launch_bounds__(256, 8) broadcast_jobs_kernel(const BroadcastJobDev *__restrict__ jobs, int njobs,
                                                             const int64_t *__restrict__ chunk0, int64_t chunks,
                                                             unsigned long long *ctr) {
    const int lane = threadIdx.x & 31;
    if (ctr) {
        for (;;) {
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(ctr, 1ull);
            const int64_t base = (int64_t)__shfl_sync(0xFFFFFFFFu, b, 0) * kBcastBatch;
            if (base >= chunks) break;
            const int64_t end = base + kBcastBatch < chunks ? base + kBcastBatch : chunks;
            int64_t c = base;
            while (c < end) {  // the batch's chunks, job by job
                const int j = ONE ? 0 : job_of(chunk0, njobs, c);
                const BroadcastJobDev &B = jobs[j];
                const int64_t first = ONE ? 0 : __ldg(chunk0 + j), last = ONE ? chunks : __ldg(chunk0 + j + 1);
                const int64_t jend = end < last ? end : last;
                if (jend <= c) break;  // (chunk0 increases: never taken)
                if ((B.w >> 1) >= 16) {  // whole rows: step (row, qubit) without dividing
                    const int hw = (int)(B.w >> 1), n = (int)B.n;
                    const int64_t lc = c - first, row = lc / n, nw64 = B.nw64;
                    int q = (int)(lc - row * n);
                    const uint64_t *xr = B.xz + row * 2 * nw64;  // the row's x bits, then its z bits
                    ulonglong2 *xo = reinterpret_cast<ulonglong2 *>(B.X + lc * B.w);
                    ulonglong2 *zo = reinterpret_cast<ulonglong2 *>(B.Z + lc * B.w);
                    // the shared bits of 64 qubits at a time: the stores of a
                    // chunk wait on no load
                    for (; c < jend; ++c) {
                        const u64 xb = (xr[q >> 6] >> (q & 63)) & 1ull, zb = (xr[nw64 + (q >> 6)] >> (q & 63)) & 1ull;
                        const ulonglong2 xv = make_ulonglong2(0ull - xb, 0ull - xb),
                                         zv = make_ulonglong2(0ull - zb, 0ull - zb);
                        for (int kp = lane; kp < hw; kp += 32) {
                            __stcs(xo + kp, xv);
                            __stcs(zo + kp, zv);
                        }
                        xo += hw;
                        zo += hw;
                        if (++q == n) {
                            q = 0;
                            xr += 2 * nw64;
                        }
                    }
                } else {
                    for (; c < jend; ++c) broadcast_chunk(B, c - first, lane);
                }
            }
        }
        __syncthreads();  // every warp of the CTA is past its last counter fetch
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(ctr + 1, 1ull) == (unsigned long long)gridDim.x - 1) {
                atomicExch(ctr, 0ull);
                atomicExch(ctr + 1, 0ull);
            }
        }
        return;
    }
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t c0 = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int64_t c = c0; c < chunks; c += warps) {
        const int j = ONE ? 0 : job_of(chunk0, njobs, c);
        broadcast_chunk(jobs[j], c - chunk0[j], lane);
    }
}

int g_frame_sms = 0;
int g_prio_greatest = 1;  // 1: not looked up yet (priorities are <= 0)
int g_prio_least = 0;

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

int prio_greatest() {
    if (g_prio_greatest == 1) {
        int least = 0, greatest = 0;
        PS_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        g_prio_least = least;
        g_prio_greatest = greatest;
    }
    return OK;
}

template <int FW>
int launch_frame_fw(cudaStream_t st, const FrameTable &t) {
    if (t.smem > 48 * 1024) {
        const int rc = allow_max_smem((const void *)frame_run_kernel<FW>);
        if (rc != OK) return rc;
    }
    int rc = same_carveout((const void *)frame_run_kernel<FW>);
    if (rc == OK) rc = prio_greatest();
    if (rc != OK) return rc;
    // The sign kernel runs at the lowest priority: it fills what the
    // broadcast's CTAs leave of each SM.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)t.ctas);
    cfg.blockDim = dim3(32 * FW);
    cfg.dynamicSmemBytes = t.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = g_prio_least;
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

int launch_noise_vectors(cudaStream_t st, const FrameTable &t) {
    if (t.njobs <= 0 || t.nctas <= 0) return OK;
    if (t.nsmem > kSegSmemMax) return fail(E_ARG, "channel noise does not fit in shared memory");
    // At most six noise CTAs an SM (8K registers each): the broadcast's two
    // CTAs (16K registers) find room beside them.
    const size_t smem = std::max<size_t>(t.nsmem, kNoiseSmemFloor);
    if (t.nctas > 0x7FFFFFFFll) return fail(E_ARG, "channel noise: too many (range, shot-word) pairs in one launch");
    const void *kern = (const void *)noise_vec_kernel<kNoiseWarps>;
    cudaLaunchConfig_t cfg;
    if (smem > 48 * 1024) {
        const int rc = allow_max_smem(kern);
        if (rc != OK) return rc;
    }
    int rc = same_carveout(kern);
    if (rc == OK) rc = prio_greatest();
    if (rc != OK) return rc;
    cfg = {};
    cfg.gridDim = dim3((unsigned)t.nctas);
    cfg.blockDim = dim3(32 * kNoiseWarps);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;  // like the sign kernel: what the broadcast leaves
    attr[0].val.priority = g_prio_least;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PS_CUDA(cudaLaunchKernelEx(&cfg, noise_vec_kernel<kNoiseWarps>, t.jobs, (int)t.njobs, t.ncta0));
    PS_CUDA(cudaGetLastError());
    return OK;
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
        int rc = same_carveout((const void *)broadcast_jobs_kernel<true>);
        if (rc == OK) rc = same_carveout((const void *)broadcast_jobs_kernel<false>);
        if (rc != OK) return rc;
    }
    int rc = prio_greatest();
    if (rc != OK) return rc;
    const int per = ctas_per_sm > 0 ? ctas_per_sm : 1;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((t.chunks + 7) / 8, (int64_t)g_frame_sms * per));
    // The broadcast is the run's longest kernel and its CTAs stay to the
    // end: launched at the highest priority, they reach every SM before the
    // noise and sign CTAs fill them.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = g_prio_greatest;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (t.njobs == 1)
        PS_CUDA(cudaLaunchKernelEx(&cfg, broadcast_jobs_kernel<true>, t.bjobs, (int)t.njobs, t.chunk0, t.chunks, t.bctr));
    else
        PS_CUDA(cudaLaunchKernelEx(&cfg, broadcast_jobs_kernel<false>, t.bjobs, (int)t.njobs, t.chunk0, t.chunks, t.bctr));
    PS_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace ps
