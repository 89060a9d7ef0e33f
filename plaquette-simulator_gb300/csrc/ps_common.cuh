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

enum : uint32_t { TAG_MEASURE = 1, TAG_NOISE = 2 };

// Draws for the 64 shots of global word `word`: block `sub` (0..15) covers
// shots 4*sub .. 4*sub+3 of the word.
PS_HD u32x4 draw_block(uint64_t seed, uint64_t event, uint64_t word, uint32_t sub, uint32_t tag) {
    return philox4x32_10(sub, (uint32_t)word, (uint32_t)event, tag, (uint32_t)(seed & 0xffffffffu),
                         (uint32_t)(seed >> 32));
}

// 24-bit uniform in [0,1), exact in binary32.
PS_HD float unit_float(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

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
