// ps_common.cuh -- shared definitions of the GB300 tableau library.
//
// Device layout of one state (n qubits, W = 2n+1 tableau rows, w shot-words
// of 64 shots each, shot index innermost):
//   X[row][qubit][word]  uint64   bit s of word k = shot 64k+s
//   Z[row][qubit][word]  uint64
//   R[row][word]         uint64
// Rows 0..n-1 are destabilizers, n..2n-1 stabilizers, 2n the scratch row,
// exactly as the reference's int32 tableau (CliffordState.hpp:66-71,
// MiscFunctors.hpp:23-27); every bit of the reference's int32 cell is one bit
// here.  A gate on qubit q touches one contiguous run of w words per row and
// plane, so every gate pass is a coalesced 128-bit stream.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>

typedef unsigned long long u64;

#define PS_HD __host__ __device__ __forceinline__

namespace ps {

// ---------------------------------------------------------------- RNG
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Round: (c0,c1,c2,c3)
// -> (hi(M1*c2)^c1^k0, lo(M1*c2), hi(M0*c0)^c3^k1, lo(M0*c0)); key bumped by
// the Weyl constants between rounds.
struct u32x4 {
    uint32_t v[4];
};

PS_HD u32x4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int round = 0; round < 10; ++round) {
#ifdef __CUDA_ARCH__
        // high and low halves as separate multiplies (measured faster here
        // than one 32x32->64 multiply)
        const uint32_t h0 = __umulhi(0xD2511F53u, c0), l0 = 0xD2511F53u * c0;
        const uint32_t h1 = __umulhi(0xCD9E8D57u, c2), l1 = 0xCD9E8D57u * c2;
#else
        const u64 p0 = (u64)0xD2511F53u * c0;
        const u64 p1 = (u64)0xCD9E8D57u * c2;
        const uint32_t h0 = (uint32_t)(p0 >> 32), l0 = (uint32_t)p0, h1 = (uint32_t)(p1 >> 32), l1 = (uint32_t)p1;
#endif
        const uint32_t n0 = h1 ^ c1 ^ k0;
        const uint32_t n1 = l1;
        const uint32_t n2 = h0 ^ c3 ^ k1;
        const uint32_t n3 = l0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    u32x4 r;
    r.v[0] = c0;
    r.v[1] = c1;
    r.v[2] = c2;
    r.v[3] = c3;
    return r;
}

enum : uint32_t { TAG_MEASURE = 1, TAG_NOISE = 2, TAG_NOISE_FIRST = 3 };

// Philox block `sub` of global word `word` for event `event`.  A random
// measurement's draws: block sub (0..15) covers shots 4*sub .. 4*sub+3 of
// the word; a Pauli channel's: see channel_word.
PS_HD u32x4 draw_block(uint64_t seed, uint64_t event, uint64_t word, uint32_t sub, uint32_t tag) {
    return philox4x32_10(sub, (uint32_t)word, (uint32_t)event, tag, (uint32_t)(seed & 0xffffffffu),
                         (uint32_t)(seed >> 32));
}

// 24-bit uniform in [0,1), exact in binary32.
PS_HD float unit_float(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

// ------------------------------------------------------ Pauli channels
// A channel's table: thr[0..count) cumulative thresholds of its Paulis
// (Pauli k+1 takes draws in [thr[k-1], thr[k]) of [0, 2^32), count 3 for
// X, Y, Z on one qubit, 15 for IX .. ZZ on two), total = thr[count-1] the
// probability p = total / 2^32 that a shot is hit, and thr[count] =
// channel_surv64(total).
//
// A shot is hit with probability p, independently of the others, and a hit
// shot takes Pauli k+1 with probability (thr[k] - thr[k-1]) / total.  The
// 64 shots of a word are sampled by their gaps: the survival products
// S_0 = 2^32, S_{j+1} = floor(S_j (2^32 - total) / 2^32) (the chance that j
// shots in a row are missed, in 32-bit fixed point: integer arithmetic, so
// every platform computes the same bits); a draw u puts the next hit g
// shots on, g the first with u >= S_{g+1}, and one more draw v picks the
// hit's Pauli as the first k with floor(v total / 2^32) < thr[k].  The first
// draw of a word is lane event%4 of the Philox block keyed by (seed,
// event/4, word, TAG_NOISE_FIRST), so one block serves the first draws of
// four consecutive channel events; draw i >= 1 is lane (i-1)%4 of block
// 1 + (i-1)/4 keyed by (seed, event, word, TAG_NOISE).  A word with no hit
// -- u < S_64 -- costs a quarter of a block.
// floor(a b / 2^32) for a, b < 2^32: the survival step S_{j+1} from S_j,
// exact for j >= 1 (S_1 = 2^32 - total < 2^32).
PS_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

PS_HD uint64_t channel_surv64(uint64_t total) {
    if (total == 0) return 1ull << 32;
    const uint32_t q = (uint32_t)((1ull << 32) - total);
    uint32_t s = q;  // S_1
    for (int j = 1; j < 64; ++j) s = mulhi32(s, q);
    return s;
}

// Lane j of a block, without indexing the block by a variable (which would
// put it in local memory).
PS_HD uint32_t block_lane(const u32x4 &b, uint32_t j) {
    return j == 0u ? b.v[0] : j == 1u ? b.v[1] : j == 2u ? b.v[2] : b.v[3];
}

struct ChannelWord {
    u64 fxa, fza, fxb, fzb;  // shots with X or Y / Y or Z on qubit a, and on qubit b
};

// The first draw of channel `event` for a word (lane event%4 of the block
// its group of four events shares).
PS_HD uint32_t channel_first_draw(uint64_t seed, uint64_t event, uint64_t word) {
    return block_lane(draw_block(seed, event >> 2, word, 0u, TAG_NOISE_FIRST), (uint32_t)(event & 3u));
}

// Later draws of a word: draw i >= 1 is lane (i-1)%4 of block 1 + (i-1)/4.
struct ChannelDraws {
    uint64_t seed, event, word;
    u32x4 blk;
    uint32_t i = 0;  // later draws taken so far
    PS_HD uint32_t next() {
        if ((i & 3u) == 0u) blk = draw_block(seed, event, word, 1u + (i >> 2), TAG_NOISE);
        return block_lane(blk, i++ & 3u);
    }
};

PS_HD void channel_set(ChannelWord &m, int pos, int idx, int count) {
    const u64 bit = 1ull << pos;
    const int pa = count == 3 ? idx : (idx >> 2), pb = count == 3 ? 0 : (idx & 3);
    if (pa == 1 || pa == 2) m.fxa |= bit;
    if (pa == 2 || pa == 3) m.fza |= bit;
    if (pb == 1 || pb == 2) m.fxb |= bit;
    if (pb == 2 || pb == 3) m.fzb |= bit;
}

PS_HD ChannelWord channel_word(uint64_t seed, uint64_t event, uint64_t word, const uint64_t *thr, int count) {
    ChannelWord m{0ull, 0ull, 0ull, 0ull};
    const uint64_t total = thr[count - 1];
    if (total == 0) return m;
    uint32_t u = channel_first_draw(seed, event, word);
    if ((uint64_t)u < thr[count]) return m;  // no shot of the word is hit
    const uint32_t q = (uint32_t)((1ull << 32) - total);
    ChannelDraws dr{seed, event, word};
    int pos = 0;  // the first shot not sampled yet
    for (;;) {
        uint32_t s = q;  // S_1
        for (;;) {       // the gap to the next hit
            if (u >= s) break;
            if (++pos == 64) return m;
            s = mulhi32(s, q);
        }
        const uint64_t v = ((uint64_t)dr.next() * total) >> 32;
        int idx = 1;
        while (v >= thr[idx - 1]) ++idx;
        channel_set(m, pos, idx, count);
        if (++pos == 64) return m;
        u = dr.next();
    }
}

// The survival products of a channel's table as a table: surv[j] = S_{j+1},
// j = 0..63, by the same integer steps channel_word takes one at a time
// (surv[63] = S_64 = thr[count]).  Unused when total = 0.
PS_HD void channel_surv_table(uint64_t total, uint32_t *surv) {
    const uint32_t q = (uint32_t)((1ull << 32) - total);
    uint32_t s = q;  // S_1
    for (int j = 0; j < 64; ++j) {
        surv[j] = s;
        s = mulhi32(s, q);
    }
}

// channel_word with the survival products read from channel_surv_table's
// table: the gap to the next hit -- the first j with u >= S_{j+1} -- is
// found by binary search (the S_j only decrease) instead of stepping S_j.
// The same outcomes bit for bit.
PS_HD ChannelWord channel_word_surv(uint64_t seed, uint64_t event, uint64_t word, const uint64_t *thr, int count,
                                    const uint32_t *surv) {
    ChannelWord m{0ull, 0ull, 0ull, 0ull};
    const uint64_t total = thr[count - 1];
    if (total == 0) return m;
    uint32_t u = channel_first_draw(seed, event, word);
    if ((uint64_t)u < thr[count]) return m;  // no shot of the word is hit
    ChannelDraws dr{seed, event, word};
    int pos = 0;  // the first shot not sampled yet
    for (;;) {
        int lo = 0, hi = 64 - pos;  // the first j in [0, 64 - pos) with u >= surv[j], else 64 - pos
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (u >= surv[mid]) hi = mid;
            else lo = mid + 1;
        }
        if (lo == 64 - pos) return m;
        pos += lo;
        const uint64_t v = ((uint64_t)dr.next() * total) >> 32;
        int idx = 1;
        while (v >= thr[idx - 1]) ++idx;
        channel_set(m, pos, idx, count);
        if (++pos == 64) return m;
        u = dr.next();
    }
}

// Float estimates for channel_word_est: the gap to the next hit is near
// log2(u / 2^32) / log2(q / 2^32) - 1 (S_{j+1} is about 2^32 (q / 2^32)^(j+1)),
// and the Pauli index near v count / total.  channel_est_factors gives the
// two factors of a table.
struct ChannelEst {
    float inv_lq;  // 1 / (log2(q) - 32), q = 2^32 - total
    float kmul;    // count / total
};
inline ChannelEst channel_est_factors(uint64_t total, int count) {
    ChannelEst e;
    const double q = 4294967296.0 - (double)total;
    e.inv_lq = q > 0.0 ? (float)(1.0 / (std::log2(q) - 32.0)) : 0.0f;
    e.kmul = total > 0 ? (float)((double)count / (double)total) : 0.0f;
    return e;
}

// Both searches of channel_word_est, started from the float estimates and
// settled on the integer tables: the first j in [0, lim) with u >= surv[j]
// (surv = channel_surv_table), and the first k with v < thr[k].  Whatever
// the estimate, the two correcting walks end on the same index as the
// stepped search, so the outcomes are channel_word's bit for bit; a close
// estimate only makes the walks short.
PS_HD int channel_first_at_least(uint32_t u, const uint32_t *surv, int lim, int g) {
    g = g < 0 ? 0 : (g > lim ? lim : g);
    while (g > 0 && u >= surv[g - 1]) --g;
    while (g < lim && u < surv[g]) ++g;
    return g;
}
PS_HD int channel_first_above(uint64_t v, const uint64_t *thr, int count, int k) {
    k = k < 0 ? 0 : (k > count - 1 ? count - 1 : k);
    while (k > 0 && v < thr[k - 1]) --k;
    while (v >= thr[k]) ++k;  // stops at count - 1 at the latest: v < total = thr[count - 1]
    return k;
}
PS_HD float channel_log2(float x) {
#ifdef __CUDA_ARCH__
    return __log2f(x);
#else
    return std::log2(x);
#endif
}

// The outcomes of a word whose first draw u hit (u >= S_64), from there on.
PS_HD ChannelWord channel_word_est_hit(uint64_t seed, uint64_t event, uint64_t word, uint32_t u, const uint64_t *thr,
                                       int count, const uint32_t *surv, ChannelEst est) {
    ChannelWord m{0ull, 0ull, 0ull, 0ull};
    const uint64_t total = thr[count - 1];
    ChannelDraws dr{seed, event, word};
    int pos = 0;  // the first shot not sampled yet
    for (;;) {
        const float L = (channel_log2((float)u) - 32.0f) * est.inv_lq;  // u = 0: +inf or NaN, clamped
        const int ge = L >= 0.0f ? (L < 80.0f ? (int)ceilf(L) - 1 : 80) : 0;
        const int lim = 64 - pos;
        const int g = channel_first_at_least(u, surv, lim, ge);
        if (g == lim) return m;
        pos += g;
        const uint64_t v = ((uint64_t)dr.next() * total) >> 32;
        const int idx = 1 + channel_first_above(v, thr, count, (int)((float)v * est.kmul));
        channel_set(m, pos, idx, count);
        if (++pos == 64) return m;
        u = dr.next();
    }
}

PS_HD ChannelWord channel_word_est(uint64_t seed, uint64_t event, uint64_t word, const uint64_t *thr, int count,
                                   const uint32_t *surv, ChannelEst est) {
    if (thr[count - 1] == 0) return ChannelWord{0ull, 0ull, 0ull, 0ull};
    const uint32_t u = channel_first_draw(seed, event, word);
    if ((uint64_t)u < thr[count]) return ChannelWord{0ull, 0ull, 0ull, 0ull};  // no shot of the word is hit
    return channel_word_est_hit(seed, event, word, u, thr, count, surv, est);
}

// ----------------------------------------------------------- sign math
// Bit-sliced mod-4 accumulation of the reference's PauliProductPhase
// (MeasurementFunctors.hpp:10-72) over 64 shots at once.  For row i (x1,z1)
// times row k (x2,z2) the phase g is +1 for XY, YZ, ZX and -1 for YX, XZ, ZY
// (first letter from row i), 0 otherwise.  (c1,c0) is a per-shot 2-bit
// counter mod 4; adding +1 / -1 is a 2-bit increment / decrement.
PS_HD void phase_accumulate(u64 x1, u64 z1, u64 x2, u64 z2, u64 mask, u64 &c1, u64 &c0) {
    const u64 plus = ((x1 & ~z1 & x2 & z2) | (x1 & z1 & ~x2 & z2) | (~x1 & z1 & x2 & ~z2)) & mask;
    const u64 minus = ((x1 & z1 & x2 & ~z2) | (x1 & ~z1 & ~x2 & z2) | (~x1 & z1 & x2 & z2)) & mask;
    c1 ^= (plus & c0) | (minus & ~c0);
    c0 ^= plus | minus;
}

// Sum of two 2-bit counters mod 4.
PS_HD void phase_add(u64 &c1, u64 &c0, u64 d1, u64 d0) {
    c1 ^= d1 ^ (c0 & d0);
    c0 ^= d0;
}

// ------------------------------------------------------------- errors
enum Status : int {
    OK = 0,
    E_ARG = 1,
    E_RANGE = 2,
    E_CUDA = 3,
    E_NOMEM = 4,
    E_STATE = 5,
    E_TIMEOUT = 6,
};

void set_error(const std::string &msg);
int fail(int status, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

} // namespace ps

#define PS_CUDA(expr)                                               \
    do {                                                            \
        cudaError_t _e = (expr);                                    \
        if (_e != cudaSuccess) return ps::cuda_fail(_e, #expr);     \
    } while (0)
