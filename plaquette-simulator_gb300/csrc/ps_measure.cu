// ps_measure.cu -- Z-basis measurement (Aaronson-Gottesman), bit-exact with
// the reference's BatchMeasureFunctor (MeasurementFunctors.hpp:267-318).
//
// One CTA owns B consecutive 64-shot words and runs a list of measurements
// ("measurement phase") in order.
//
// Windows of deterministic measurements.  A deterministic measurement only
// rewrites the scratch row 2n (MeasureDetermined, :189-201); rows 0..2n-1,
// which decide whether a later measurement is random and which rows it
// multiplies, stay unchanged.  So a window of up to 16 measurements is
// scanned at once, one warp per measurement (column q of all 2n rows:
// no stabilizer row with x(.,q)=1 means deterministic; the destabilizer rows
// with x(i,q)=1 select the stabilizer rows i+n to multiply).  The leading run
// of deterministic measurements is then computed concurrently, one warp each:
// the product's sign follows the reference's step order exactly (per-step
// phase sums, bit 1 of each, :97-129), and only the last measurement of the
// run writes the scratch row -- the value the sequential order leaves there.
//
// Everything else (a measurement that is random for some shot, more than
// KMAX rows to multiply, or a reset whose X must act before the next
// measurement) runs on the whole CTA:
//  - column q is staged in shared memory; warp b finds for word b the lowest
//    stabilizer row p+n with x(p+n,q)=1 per shot (ballot + ffs, :297-301);
//  - if every shot of every word takes the random branch with the same pivot
//    (the usual case), MeasureRandom (:225-265) runs once for all B words:
//    row p+n copied to row p, row p+n := +-Z_q with the drawn outcome, and
//    every row i != p, p+n with x(i,q)=1 multiplied by the copied row (one
//    warp per row, lanes over (column, word), bit-sliced mod-4 phase
//    counters reduced with shuffles);
//  - otherwise each word is processed alone with per-shot pivot groups and an
//    exact deterministic branch for the shots without a pivot.
#include <vector>

#include "ps_internal.h"
#include "ps_segment.cuh"
#include "ps_draw.cuh"

namespace ps {

namespace {

constexpr int NW = 16;          // warps per CTA = measurements per window
constexpr int KMAX = 8;         // rows per deterministic measurement in the warp path
constexpr int MAXC = 4;         // columns per thread in the single-word deterministic branch
constexpr int STEP_CHUNK = 32;  // deterministic steps reduced per round (single-word branch)

enum : int { ST_DET = 0, ST_DET_RESET = 1, ST_OTHER = 2 };

struct Ctl {
    int status[NW];
    int kcnt[NW];
    int ngroups[4];
    int gp[4][64];
    u64 gm[4][64];
    u64 det_mask[4];
    u64 outcome[4];
    u64 res[4];
    u64 detw[4];
    u64 pr[4];
    u64 racc;
    int cnt;
    int uniform;
    int rows_done;
    int resq[NW];  // window slot -> qubit of its reset, or -1
    MeasOp wop[NW];  // the window's measurements
    int miss[NW];    // the slot scanned its column (not found in the scan cache)
    int epoch;       // scan-cache epoch: advanced by every measurement on the CTA-wide path
};
// Dynamic shared memory a measurement launch may take: the opt-in maximum
// less the kernel's static control block.
constexpr size_t kMeasSmemMax = 227 * 1024 - sizeof(Ctl) - 256;


struct Smem {
    u64 *col;      // [2n][B]
    u64 *prow;     // [2][n][B]
    u64 *part;     // [STEP_CHUNK][NW][2]
    int *rowlist;  // [2n]
    int *klist;    // [NW][KMAX]
    u64 *kmask;    // [NW][KMAX][B]
    u64 *wraw;     // [NW][B] window outcomes before reset corrections
    u64 *wres;     // [NW][B] window outcomes
    u64 *wz;       // [NW][NW][B] z of measurement j's product row at reset r's qubit
    // Scan cache (optional): per qubit, the last deterministic scan of its
    // column -- rows to multiply and their per-word masks -- valid while its
    // tag equals the epoch.  Deterministic measurements and resets leave x
    // and z of rows < 2n unchanged, so a scan stays valid until a measurement
    // runs on the CTA-wide path (a random one rewrites rows).
    u64 *ckmask;   // [n][KMAX][B]
    int *cmeta;    // [n][2 + KMAX]: tag, row count, rows
};

__device__ __forceinline__ void warp_phase_reduce(u64 &c1, u64 &c0, int first_offset) {
    for (int off = 16; off >= first_offset; off >>= 1) {
        const u64 d1 = __shfl_xor_sync(0xffffffffu, c1, off);
        const u64 d0 = __shfl_xor_sync(0xffffffffu, c0, off);
        phase_add(c1, c0, d1, d0);
    }
}


// B consecutive shot-words of one (row, column) cell, loaded as one vector.
template <int B> struct Cell {
    u64 v[B];
};
template <int B> __device__ __forceinline__ Cell<B> load_cell(const u64 *p) {
    Cell<B> c;
    if (B == 1) {
        c.v[0] = *p;
    } else {
#pragma unroll
        for (int h = 0; h < B / 2; ++h) {
            const ulonglong2 t = reinterpret_cast<const ulonglong2 *>(p)[h];
            c.v[2 * h] = t.x;
            c.v[2 * h + 1] = t.y;
        }
    }
    return c;
}
template <int B> __device__ __forceinline__ void store_cell(u64 *p, const u64 *v) {
    if (B == 1) {
        *p = v[0];
    } else {
#pragma unroll
        for (int h = 0; h < B / 2; ++h)
            reinterpret_cast<ulonglong2 *>(p)[h] = make_ulonglong2(v[2 * h], v[2 * h + 1]);
    }
}

// Warp scan of column q for the window path: lane = row, each lane loads the
// B words of its row's cell.  Returns ST_DET / ST_DET_RESET / ST_OTHER and
// fills this warp's ordered row list (klist) and per-word masks (kmask).
template <int B>
__device__ int warp_scan(const u64 *X, int64_t n, int64_t w, int64_t k0, const MeasOp &op, int *klist, u64 *kmask,
                         int &kcnt_out) {
    constexpr int U = 32 / B;  // rows in flight per lane (32 words per lane)
    const int lane = threadIdx.x & 31;
    const int64_t q = op.q;
    u64 stab[B];
#pragma unroll
    for (int bb = 0; bb < B; ++bb) stab[bb] = 0ull;
    int kcnt = 0;
    for (int64_t i0 = 0; i0 < 2 * n; i0 += 32 * U) {
        Cell<B> c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = i0 + (int64_t)u * 32 + lane;
            if (i < 2 * n) {
                c[u] = load_cell<B>(X + (i * n + q) * w + k0);
            } else {
#pragma unroll
                for (int bb = 0; bb < B; ++bb) c[u].v[bb] = 0ull;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = i0 + (int64_t)u * 32 + lane;
            const bool stab_row = i >= n;
            bool hit = false;
#pragma unroll
            for (int bb = 0; bb < B; ++bb) {
                if (stab_row) stab[bb] |= c[u].v[bb];
                hit |= !stab_row && c[u].v[bb] != 0ull;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, hit);
            if (hit) {
                const int pos = kcnt + __popc(bal & ((1u << lane) - 1u));
                if (pos < KMAX) {
                    klist[pos] = (int)i;
#pragma unroll
                    for (int bb = 0; bb < B; ++bb) kmask[pos * B + bb] = c[u].v[bb];
                }
            }
            kcnt += __popc(bal);
        }
    }
    bool random = false;
#pragma unroll
    for (int bb = 0; bb < B; ++bb) random |= stab[bb] != 0ull;
    random = __ballot_sync(0xffffffffu, random) != 0u;
    kcnt_out = kcnt;
    if (random || kcnt > KMAX) return ST_OTHER;
    return op.reset ? ST_DET_RESET : ST_DET;
}

// Deterministic measurement of all B words by one warp (rows from warp_scan,
// at most KR of them).  Lane = (column slot, word): 32/B columns per
// instruction, UC column groups of all rows in flight together.  If
// `writer`, the product becomes the scratch row.
template <int B, int KR, int UC>
__device__ void warp_det_rows(u64 *X, u64 *Z, const u64 *R, int64_t n, int64_t w, int64_t k0, const int *klist,
                              const u64 *kmask, int kp, bool writer, int slot, const int *resq, u64 *wraw,
                              u64 *wz) {
    constexpr int CPI = 32 / B;
    const int lane = threadIdx.x & 31, cs = lane / B, b = lane % B;
    const int64_t k = k0 + b;
    const int64_t srow = 2 * n * n;
    u64 c1[KR], c0[KR], m[KR];
    int64_t ro[KR];
#pragma unroll
    for (int t = 0; t < KR; ++t) {
        c1[t] = c0[t] = 0ull;
        m[t] = t < kp ? kmask[t * B + b] : 0ull;
        ro[t] = t < kp ? ((int64_t)klist[t] + n) * n : 0;
    }
    for (int64_t j0 = cs; j0 < n; j0 += (int64_t)CPI * UC) {
        u64 xr[UC][KR], zr[UC][KR];
#pragma unroll
        for (int uc = 0; uc < UC; ++uc) {
            const int64_t j = j0 + (int64_t)uc * CPI;
#pragma unroll
            for (int t = 0; t < KR; ++t) {
                const bool ok = t < kp && j < n;
                xr[uc][t] = ok ? X[(ro[t] + j) * w + k] : 0ull;
                zr[uc][t] = ok ? Z[(ro[t] + j) * w + k] : 0ull;
            }
        }
#pragma unroll
        for (int uc = 0; uc < UC; ++uc) {
            const int64_t j = j0 + (int64_t)uc * CPI;
            u64 ax = 0ull, az = 0ull;
#pragma unroll
            for (int t = 0; t < KR; ++t) {
                phase_accumulate(ax, az, xr[uc][t], zr[uc][t], m[t], c1[t], c0[t]);
                ax ^= xr[uc][t] & m[t];
                az ^= zr[uc][t] & m[t];
            }
            if (writer && j < n) {
                X[(srow + j) * w + k] = ax;
                Z[(srow + j) * w + k] = az;
            }
        }
    }
    u64 racc = 0ull;
#pragma unroll
    for (int t = 0; t < KR; ++t)
        if (t < kp) {
            warp_phase_reduce(c1[t], c0[t], B);
            racc ^= (R[((int64_t)klist[t] + n) * w + k] ^ c1[t]) & m[t];
        }
    if (cs == 0) wraw[slot * B + b] = racc;
    // z of the product row at the qubit of each earlier reset in the window
    // (lane = (earlier slot mod CPI, word)): a reset's X flips the sign of every row
    // with z on its qubit, so it flips this outcome where that z is set.
    for (int rr = cs; rr < slot; rr += CPI) {
        if (resq[rr] < 0) continue;
        const int64_t qr = resq[rr];
        u64 zb = 0ull;
#pragma unroll
        for (int t = 0; t < KR; ++t)
            if (t < kp) zb ^= Z[(ro[t] + qr) * w + k] & m[t];
        wz[(slot * NW + rr) * B + b] = zb;
    }
}

template <int B>
__device__ void warp_det(u64 *X, u64 *Z, const u64 *R, int64_t n, int64_t w, int64_t k0, const int *klist,
                         const u64 *kmask, int kp, bool writer, int slot, const int *resq, u64 *wraw, u64 *wz) {
    if (kp <= 1)
        warp_det_rows<B, 1, 8>(X, Z, R, n, w, k0, klist, kmask, kp, writer, slot, resq, wraw, wz);
    else if (kp <= 2)
        warp_det_rows<B, 2, 4>(X, Z, R, n, w, k0, klist, kmask, kp, writer, slot, resq, wraw, wz);
    else if (kp <= 4)
        warp_det_rows<B, 4, 2>(X, Z, R, n, w, k0, klist, kmask, kp, writer, slot, resq, wraw, wz);
    else
        warp_det_rows<B, KMAX, 1>(X, Z, R, n, w, k0, klist, kmask, kp, writer, slot, resq, wraw, wz);
}

// ---------------------------------------------------------------------------
// CTA-wide paths.

// Single word, any tableau: per-shot pivot groups + exact deterministic
// branch (the sequential algorithm with 64 shots bit-sliced).
template <int B>
__device__ void cta_word(u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, int64_t k0, int b, const MeasOp &op,
                         const Smem &s, Ctl &ctl, uint64_t seed, uint64_t event_base) {
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = T >> 5;
    const int64_t k = k0 + b;
    const int64_t q = op.q;
    u64 *col = s.col;  // strided by B: col[i*B + b]
    u64 *prow_x = s.prow, *prow_z = s.prow + n * B;  // word-local use: [j*B + b]
    const int ng = ctl.ngroups[b];
    const u64 outcome = ctl.outcome[b];
    u64 res_word = 0ull;
    for (int g = 0; g < ng; ++g) {
        const int64_t p = ctl.gp[b][g];
        const u64 mm = ctl.gm[b][g];
        for (int64_t j = tid; j < n; j += T) {
            prow_x[j * B + b] = X[((p + n) * n + j) * w + k];
            prow_z[j * B + b] = Z[((p + n) * n + j) * w + k];
        }
        if (tid == 0) {
            ctl.pr[b] = R[(p + n) * w + k];
            ctl.cnt = 0;
        }
        __syncthreads();
        const u64 pr = ctl.pr[b];
        for (int64_t j = tid; j < n; j += T) {
            const int64_t o = (p * n + j) * w + k, o2 = ((p + n) * n + j) * w + k;
            X[o] = (X[o] & ~mm) | (prow_x[j * B + b] & mm);
            Z[o] = (Z[o] & ~mm) | (prow_z[j * B + b] & mm);
            X[o2] &= ~mm;
            Z[o2] = (Z[o2] & ~mm) | (j == q ? mm : 0ull);
        }
        if (tid == 0) {
            R[p * w + k] = (R[p * w + k] & ~mm) | (pr & mm);
            R[(p + n) * w + k] = (R[(p + n) * w + k] & ~mm) | (outcome & mm);
        }
        for (int64_t i = tid; i < 2 * n; i += T)
            if (i != p && i != p + n && (col[i * B + b] & mm)) s.rowlist[atomicAdd(&ctl.cnt, 1)] = (int)i;
        __syncthreads();
        const int cnt = ctl.cnt;
        if (tid == 0) ctl.rows_done += cnt;
        for (int t = warp; t < cnt; t += nwarps) {
            const int64_t i = s.rowlist[t];
            const u64 mi = col[i * B + b] & mm;
            u64 c1 = 0ull, c0 = 0ull;
            for (int64_t j = lane; j < n; j += 32) {
                const int64_t o = (i * n + j) * w + k;
                const u64 xi = X[o], zi = Z[o], xp = prow_x[j * B + b], zp = prow_z[j * B + b];
                phase_accumulate(xi, zi, xp, zp, mi, c1, c0);
                X[o] = xi ^ (xp & mi);
                Z[o] = zi ^ (zp & mi);
            }
            warp_phase_reduce(c1, c0, 1);
            if (lane == 0) {
                const u64 ri = R[i * w + k];
                R[i * w + k] = (ri & ~mi) | ((ri ^ pr ^ c1) & mi);
            }
        }
        res_word |= outcome & mm;
        __syncthreads();
    }
    const u64 dm = ctl.det_mask[b];
    if (dm) {
        if (warp == 0) {
            int cnt = 0;
            for (int64_t base = 0; base < n; base += 32) {
                const int64_t i = base + lane;
                const bool v = i < n && (col[i * B + b] & dm);
                const unsigned bal = __ballot_sync(0xffffffffu, v);
                if (v) s.rowlist[cnt + __popc(bal & ((1u << lane) - 1u))] = (int)i;
                cnt += __popc(bal);
            }
            if (lane == 0) {
                ctl.cnt = cnt;
                ctl.racc = 0ull;
                ctl.rows_done += cnt;
            }
        }
        __syncthreads();
        const int cnt = ctl.cnt;
        u64 ax[MAXC], az[MAXC];
#pragma unroll
        for (int u = 0; u < MAXC; ++u) ax[u] = az[u] = 0ull;
        for (int c0s = 0; c0s < cnt; c0s += STEP_CHUNK) {
            const int len = min(STEP_CHUNK, cnt - c0s);
            for (int t = 0; t < len; ++t) {
                const int64_t i = s.rowlist[c0s + t];
                const u64 mt = col[i * B + b] & dm;
                const int64_t srow = i + n;
                u64 c1 = 0ull, c0 = 0ull;
#pragma unroll
                for (int u = 0; u < MAXC; ++u) {
                    const int64_t j = tid + (int64_t)u * T;
                    if (j < n) {
                        const int64_t o = (srow * n + j) * w + k;
                        const u64 xr = X[o], zr = Z[o];
                        phase_accumulate(ax[u], az[u], xr, zr, mt, c1, c0);
                        ax[u] ^= xr & mt;
                        az[u] ^= zr & mt;
                    }
                }
                warp_phase_reduce(c1, c0, 1);
                if (lane == 0) {
                    s.part[(t * nwarps + warp) * 2] = c1;
                    s.part[(t * nwarps + warp) * 2 + 1] = c0;
                }
            }
            __syncthreads();
            if (tid < len) {
                const int t = tid;
                u64 s1 = 0ull, s0 = 0ull;
                for (int wv = 0; wv < nwarps; ++wv)
                    phase_add(s1, s0, s.part[(t * nwarps + wv) * 2], s.part[(t * nwarps + wv) * 2 + 1]);
                const int64_t i = s.rowlist[c0s + t];
                const u64 mt = col[i * B + b] & dm;
                atomicXor(&ctl.racc, (R[(i + n) * w + k] ^ s1) & mt);
            }
            __syncthreads();
        }
        const int64_t srow = 2 * n;
#pragma unroll
        for (int u = 0; u < MAXC; ++u) {
            const int64_t j = tid + (int64_t)u * T;
            if (j < n) {
                const int64_t o = (srow * n + j) * w + k;
                X[o] = (X[o] & ~dm) | ax[u];
                Z[o] = (Z[o] & ~dm) | az[u];
            }
        }
        const u64 racc = ctl.racc;
        if (tid == 0) R[srow * w + k] = (R[srow * w + k] & ~dm) | racc;
        res_word |= racc & dm;
    }
    if (tid == 0) {
        ctl.res[b] = res_word;
        ctl.detw[b] = dm;
    }
    __syncthreads();
}

// All B words share one pivot p and every shot is random: MeasureRandom once
// for the B words.
template <int B>
__device__ void cta_uniform_random(u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, int64_t k0, const MeasOp &op,
                                   const Smem &s, Ctl &ctl) {
    constexpr int CPI = 32 / B;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = T >> 5;
    const int64_t p = ctl.gp[0][0];
    const int64_t q = op.q;
    u64 *prow_x = s.prow, *prow_z = s.prow + n * B;
    constexpr int CB = 2;  // cells in flight per thread
    for (int64_t e0 = tid; e0 < n * B; e0 += (int64_t)CB * T) {
        u64 vx[CB], vz[CB];
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            const int64_t e = e0 + (int64_t)c * T;
            const bool ok = e < n * B;
            const int64_t o2 = ((p + n) * n + e / B) * w + k0 + e % B;
            vx[c] = ok ? X[o2] : 0ull;
            vz[c] = ok ? Z[o2] : 0ull;
        }
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            const int64_t e = e0 + (int64_t)c * T;
            if (e < n * B) {
                prow_x[e] = vx[c];
                prow_z[e] = vz[c];
            }
        }
    }
    if (tid < B) ctl.pr[tid] = R[(p + n) * w + k0 + tid];
    if (tid == 0) ctl.cnt = 0;
    __syncthreads();
    // row p := old row p+n, row p+n := Z_q (masked to the shots of the pivot)
    for (int64_t e0 = tid; e0 < n * B; e0 += (int64_t)CB * T) {
        u64 xo[CB], zo[CB], xo2[CB], zo2[CB];
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            const int64_t e = e0 + (int64_t)c * T;
            const bool ok = e < n * B;
            const int64_t j = e / B, kk = k0 + e % B;
            const int64_t o = (p * n + j) * w + kk, o2 = ((p + n) * n + j) * w + kk;
            xo[c] = ok ? X[o] : 0ull;
            zo[c] = ok ? Z[o] : 0ull;
            xo2[c] = ok ? X[o2] : 0ull;
            zo2[c] = ok ? Z[o2] : 0ull;
        }
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            const int64_t e = e0 + (int64_t)c * T;
            if (e >= n * B) continue;
            const int64_t j = e / B;
            const int bb = (int)(e % B);
            const u64 mm = ctl.gm[bb][0];
            const int64_t o = (p * n + j) * w + k0 + bb, o2 = ((p + n) * n + j) * w + k0 + bb;
            X[o] = (xo[c] & ~mm) | (prow_x[e] & mm);
            Z[o] = (zo[c] & ~mm) | (prow_z[e] & mm);
            X[o2] = xo2[c] & ~mm;
            Z[o2] = (zo2[c] & ~mm) | (j == q ? mm : 0ull);
        }
    }
    if (tid < B) {
        const int bb = tid;
        const u64 mm = ctl.gm[bb][0];
        const int64_t k = k0 + bb;
        R[p * w + k] = (R[p * w + k] & ~mm) | (ctl.pr[bb] & mm);
        R[(p + n) * w + k] = (R[(p + n) * w + k] & ~mm) | (ctl.outcome[bb] & mm);
    }
    for (int64_t i = tid; i < 2 * n; i += T) {
        if (i == p || i == p + n) continue;
        bool any = false;
#pragma unroll
        for (int bb = 0; bb < B; ++bb) any |= (s.col[i * B + bb] & ctl.gm[bb][0]) != 0ull;
        if (any) s.rowlist[atomicAdd(&ctl.cnt, 1)] = (int)i;
    }
    __syncthreads();
    const int cnt = ctl.cnt;
    const int cs = lane / B, b = lane % B;
    const int64_t k = k0 + b;
    const u64 mw = ctl.gm[b][0];
    // Work items: (row, column slice).  With few rows each row is split over
    // several warps; partial phase counters meet in shared memory.
    const int slices = cnt >= nwarps ? 1 : max(1, nwarps / max(cnt, 1));
    const int64_t slice_len = ((n + slices - 1) / slices + CPI - 1) / CPI * CPI;
    const int cap = STEP_CHUNK * NW / B;  // items whose partials fit in s.part
    for (int c0i = 0; c0i < cnt * slices; c0i += cap) {
        const int c1i = min(cnt * slices, c0i + cap);
        for (int item = c0i + warp; item < c1i; item += nwarps) {
            const int t = item / slices, sl = item % slices;
            const int64_t i = s.rowlist[t];
            const u64 mi = s.col[i * B + b] & mw;
            const int64_t jb = (int64_t)sl * slice_len, je = min(n, jb + slice_len);
            u64 c1 = 0ull, c0 = 0ull;
            constexpr int UR = 8;
            for (int64_t j0 = jb + cs; j0 < je; j0 += (int64_t)CPI * UR) {
                u64 xi[UR], zi[UR];
#pragma unroll
                for (int u = 0; u < UR; ++u) {
                    const int64_t j = j0 + (int64_t)u * CPI;
                    xi[u] = j < je ? X[(i * n + j) * w + k] : 0ull;
                    zi[u] = j < je ? Z[(i * n + j) * w + k] : 0ull;
                }
#pragma unroll
                for (int u = 0; u < UR; ++u) {
                    const int64_t j = j0 + (int64_t)u * CPI;
                    if (j < je) {
                        const u64 xp = prow_x[j * B + b], zp = prow_z[j * B + b];
                        phase_accumulate(xi[u], zi[u], xp, zp, mi, c1, c0);
                        if (mi) {
                            X[(i * n + j) * w + k] = xi[u] ^ (xp & mi);
                            Z[(i * n + j) * w + k] = zi[u] ^ (zp & mi);
                        }
                    }
                }
            }
            warp_phase_reduce(c1, c0, B);
            if (cs == 0) {
                s.part[((item - c0i) * B + b) * 2] = c1;
                s.part[((item - c0i) * B + b) * 2 + 1] = c0;
            }
        }
        __syncthreads();
        // rows whose every slice lies in this chunk of items
        const int t0 = (c0i + slices - 1) / slices, t1 = c1i / slices;
        for (int e = t0 * B + tid; e < t1 * B; e += T) {
            const int t = e / B, bb = e % B;
            const int64_t i = s.rowlist[t];
            const u64 mi = s.col[i * B + bb] & ctl.gm[bb][0];
            u64 s1 = 0ull, s0 = 0ull;
            for (int sl = 0; sl < slices; ++sl) {
                const int it = t * slices + sl - c0i;
                phase_add(s1, s0, s.part[(it * B + bb) * 2], s.part[(it * B + bb) * 2 + 1]);
            }
            if (mi) {
                const u64 ri = R[i * w + k0 + bb];
                R[i * w + k0 + bb] = (ri & ~mi) | ((ri ^ ctl.pr[bb] ^ s1) & mi);
            }
        }
        __syncthreads();
    }
    if (tid < B) {
        ctl.res[tid] = ctl.outcome[tid] & ctl.gm[tid][0];
        ctl.detw[tid] = 0ull;
    }
    if (tid == 0) ctl.rows_done += cnt;
    __syncthreads();
}

// Every shot of every word deterministic (MeasureDetermined, :189-201) with
// many rows: all warps share the measurement, split over columns; the rows
// are stepped SC at a time with all their loads in flight, and each step's
// phase sum meets in shared memory (reference step order kept exactly).
template <int B, int MAXE>
__device__ void cta_det(u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, int64_t k0, const Smem &s, Ctl &ctl) {
    constexpr int SC = 16 / MAXE;  // steps in flight; MAXE = cells (column, word) per thread
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = T >> 5;
    const int b = tid % B;   // T is a multiple of B: a thread's cells share one word
    if (warp == 0) {
        int cnt = 0;
        for (int64_t base = 0; base < n; base += 32) {
            const int64_t i = base + lane;
            bool v = false;
            if (i < n)
#pragma unroll
                for (int bb = 0; bb < B; ++bb) v |= s.col[i * B + bb] != 0ull;
            const unsigned bal = __ballot_sync(0xffffffffu, v);
            if (v) s.rowlist[cnt + __popc(bal & ((1u << lane) - 1u))] = (int)i;
            cnt += __popc(bal);
        }
        if (lane == 0) ctl.cnt = cnt;
    }
    if (tid < B) ctl.res[tid] = 0ull;
    __syncthreads();
    const int cnt = ctl.cnt;
    if (tid == 0) ctl.rows_done += cnt;
    u64 ax[MAXE], az[MAXE];
    int64_t cell[MAXE];
#pragma unroll
    for (int u = 0; u < MAXE; ++u) {
        ax[u] = az[u] = 0ull;
        const int64_t e = tid + (int64_t)u * T;
        cell[u] = e < n * B ? (e / B) * w + k0 + b : -1;  // column offset within a row
    }
    for (int s0 = 0; s0 < cnt; s0 += SC) {
        const int ks = min(SC, cnt - s0);
        u64 xr[SC][MAXE], zr[SC][MAXE];
#pragma unroll
        for (int t = 0; t < SC; ++t) {
            const int64_t ro = t < ks ? ((int64_t)s.rowlist[s0 + t] + n) * n * w : 0;
#pragma unroll
            for (int u = 0; u < MAXE; ++u) {
                const bool ok = t < ks && cell[u] >= 0;
                xr[t][u] = ok ? X[ro + cell[u]] : 0ull;
                zr[t][u] = ok ? Z[ro + cell[u]] : 0ull;
            }
        }
#pragma unroll
        for (int t = 0; t < SC; ++t) {
            if (t >= ks) break;
            const u64 mt = s.col[(int64_t)s.rowlist[s0 + t] * B + b];
            u64 c1 = 0ull, c0 = 0ull;
#pragma unroll
            for (int u = 0; u < MAXE; ++u) {
                phase_accumulate(ax[u], az[u], xr[t][u], zr[t][u], mt, c1, c0);
                ax[u] ^= xr[t][u] & mt;
                az[u] ^= zr[t][u] & mt;
            }
            warp_phase_reduce(c1, c0, B);
            if (lane < B) {
                s.part[((t * nwarps + warp) * B + b) * 2] = c1;
                s.part[((t * nwarps + warp) * B + b) * 2 + 1] = c0;
            }
        }
        __syncthreads();
        if (tid < ks * B) {
            const int t = tid / B, bb = tid % B;
            u64 s1 = 0ull, sz = 0ull;
            for (int wv = 0; wv < nwarps; ++wv)
                phase_add(s1, sz, s.part[((t * nwarps + wv) * B + bb) * 2], s.part[((t * nwarps + wv) * B + bb) * 2 + 1]);
            const int64_t i = s.rowlist[s0 + t];
            const u64 mt = s.col[i * B + bb];
            atomicXor(&ctl.res[bb], (R[(i + n) * w + k0 + bb] ^ s1) & mt);
        }
        __syncthreads();
    }
    const int64_t srow = 2 * n * n * w;
#pragma unroll
    for (int u = 0; u < MAXE; ++u)
        if (cell[u] >= 0) {
            X[srow + cell[u]] = ax[u];
            Z[srow + cell[u]] = az[u];
        }
    if (tid < B) {
        R[2 * n * w + k0 + tid] = ctl.res[tid];
        ctl.detw[tid] = ~0ull;
    }
    __syncthreads();
}

// One measurement on the whole CTA (all B words).
template <int B>
__device__ void cta_measure(u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, int64_t k0, const MeasOp &op,
                            const Smem &s, Ctl &ctl, uint64_t seed, uint64_t event_base, uint64_t word_base) {
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t q = op.q;
    {
        // column q of all 2n rows, CB loads in flight per thread
        constexpr int CB = 4;
        for (int64_t e0 = tid; e0 < 2 * n * B; e0 += (int64_t)CB * T) {
            u64 v[CB];
#pragma unroll
            for (int c = 0; c < CB; ++c) {
                const int64_t e = e0 + (int64_t)c * T;
                v[c] = e < 2 * n * B ? X[((e / B) * n + q) * w + k0 + (e % B)] : 0ull;
            }
#pragma unroll
            for (int c = 0; c < CB; ++c) {
                const int64_t e = e0 + (int64_t)c * T;
                if (e < 2 * n * B) s.col[e] = v[c];
            }
        }
    }
    if (tid == 0) ctl.rows_done = 0;
    __syncthreads();
    if (warp < B) {
        const int b = warp;
        u64 rem = ~0ull;
        int ng = 0;
        int64_t p0 = 0;
        while (rem && p0 < n) {
            bool found = false;
            for (int64_t base = p0; base < n; base += 32) {
                const int64_t p = base + lane;
                const u64 v = (p < n) ? (s.col[(n + p) * B + b] & rem) : 0ull;
                const unsigned bal = __ballot_sync(0xffffffffu, v != 0ull);
                if (bal) {
                    const int f = __ffs(bal) - 1;
                    const u64 hit = __shfl_sync(0xffffffffu, v, f);
                    if (lane == 0) {
                        ctl.gp[b][ng] = (int)(base + f);
                        ctl.gm[b][ng] = hit;
                    }
                    ++ng;
                    rem &= ~hit;
                    p0 = base + f + 1;
                    found = true;
                    break;
                }
            }
            if (!found) break;
        }
        const u64 bits = ng > 0 ? outcome_bits(op, lane, seed, event_base, k0 + b, word_base) : 0ull;
        if (lane == 0) {
            ctl.ngroups[b] = ng;
            ctl.det_mask[b] = rem;
            ctl.outcome[b] = bits;
        }
    }
    __syncthreads();
    if (tid == 0) {
        int uni = 1;
        for (int bb = 0; bb < B; ++bb)
            uni &= ctl.ngroups[bb] == 1 && ctl.det_mask[bb] == 0ull && ctl.gp[bb][0] == ctl.gp[0][0];
        ctl.uniform = uni;
    }
    __syncthreads();
    bool all_det = true;
    for (int bb = 0; bb < B; ++bb) all_det &= ctl.ngroups[bb] == 0;
    const int64_t cells = (int64_t)B * n;
    if (all_det && cells <= T) {
        cta_det<B, 1>(X, Z, R, n, w, k0, s, ctl);
    } else if (all_det && cells <= 2 * T) {
        cta_det<B, 2>(X, Z, R, n, w, k0, s, ctl);
    } else if (all_det && cells <= 4 * T) {
        cta_det<B, 4>(X, Z, R, n, w, k0, s, ctl);
    } else if (ctl.uniform) {
        cta_uniform_random<B>(X, Z, R, n, w, k0, op, s, ctl);
    } else {
        for (int b = 0; b < B; ++b) cta_word<B>(X, Z, R, n, w, k0, b, op, s, ctl, seed, event_base);
    }
    if (tid < B) {
        op.res[k0 + tid] = ctl.res[tid];
        op.det[k0 + tid] = ctl.detw[tid];
    }
    if (tid == 0 && op.kstat && k0 == 0) {
        op.kstat[0] = ctl.ngroups[0] > 0;
        op.kstat[1] = ctl.rows_done;
    }
    __syncthreads();
}

// X on the shots whose outcome is 1 (ResetQubit): rows with Z on q flip sign.
template <int B>
__device__ void cta_reset_flip(const u64 *Z, u64 *R, int64_t n, int64_t w, int64_t k0, const MeasOp &op) {
    const int T = blockDim.x, tid = threadIdx.x;
    const int64_t W = 2 * n + 1;
    for (int64_t e = tid; e < W * B; e += T) {
        const int64_t i = e / B;
        const int64_t k = k0 + e % B;
        R[i * w + k] ^= op.res[k] & Z[(i * n + op.q) * w + k];
    }
    __syncthreads();
}

template <int B>
__global__ void __launch_bounds__(NW * 32, 1) measure_kernel(u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w,
                                                            const MeasOp *__restrict__ ops, int nops,
                                                            uint64_t seed_arg, uint64_t word_base_arg,
                                                            const RunParams *__restrict__ rp,
                                                            int window_max, int use_cache) {
    extern __shared__ u64 dyn[];
    __shared__ Ctl ctl;
    const uint64_t seed = rp ? rp->seed : seed_arg;
    const uint64_t event_base = rp ? rp->event_base : 0ull;
    const uint64_t word_base = rp ? rp->word_base : word_base_arg;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int64_t k0 = (int64_t)blockIdx.x * B;
    Smem s;
    s.col = dyn;
    s.prow = s.col + 2 * n * B;
    s.part = s.prow + 2 * n * B;
    s.kmask = s.part + STEP_CHUNK * NW * 2;
    s.wraw = s.kmask + NW * KMAX * B;
    s.wres = s.wraw + NW * B;
    s.wz = s.wres + NW * B;
    s.ckmask = s.wz + NW * NW * B;
    s.rowlist = reinterpret_cast<int *>(s.ckmask + (use_cache ? n * KMAX * B : 0));
    s.klist = s.rowlist + 2 * n;
    s.cmeta = s.klist + NW * KMAX;
    constexpr int CM = 2 + KMAX;  // ints per qubit in cmeta

    int pos = 0;
    if (window_max <= 0) {
        // No window: every measurement on the whole CTA (single-op launches).
        for (; pos < nops; ++pos) {
            const MeasOp op = ops[pos];
            cta_measure<B>(X, Z, R, n, w, k0, op, s, ctl, seed, event_base, word_base);
            if (op.reset) cta_reset_flip<B>(Z, R, n, w, k0, op);
        }
        return;
    }
    if (use_cache) {
        for (int64_t q = tid; q < n; q += blockDim.x) s.cmeta[q * CM] = -1;
        if (tid == 0) ctl.epoch = 0;
        __syncthreads();
    }
    int window = window_max > NW ? NW : window_max;
    while (pos < nops) {
        const int act = min(window, nops - pos);
        if (warp < act) {
            const int lane = tid & 31;
            const MeasOp op = ops[pos + warp];
            int kc = 0, st;
            const int *cm = use_cache ? s.cmeta + (int64_t)op.q * CM : nullptr;
            const bool hit = use_cache && cm[0] == ctl.epoch;
            if (hit) {  // the column's rows are still the ones a scan found
                kc = cm[1];
                if (lane < KMAX) s.klist[warp * KMAX + lane] = cm[2 + lane];
                if (lane < KMAX * B) s.kmask[warp * KMAX * B + lane] = s.ckmask[(int64_t)op.q * KMAX * B + lane];
                st = op.reset ? ST_DET_RESET : ST_DET;
                __syncwarp();
            } else {
                st = warp_scan<B>(X, n, w, k0, op, s.klist + warp * KMAX, s.kmask + warp * KMAX * B, kc);
            }
            if (lane == 0) {
                ctl.status[warp] = st;
                ctl.kcnt[warp] = kc;
                ctl.wop[warp] = op;
                ctl.miss[warp] = !hit;
            }
        }
        __syncthreads();
        // Fresh deterministic scans into the cache (read from the next
        // window on, after the barriers that follow).
        if (use_cache && warp < act && ctl.miss[warp] && ctl.status[warp] != ST_OTHER) {
            const int lane = tid & 31;
            const int64_t q = ctl.wop[warp].q;
            int *cm = s.cmeta + q * CM;
            if (lane < KMAX) cm[2 + lane] = s.klist[warp * KMAX + lane];
            if (lane < KMAX * B) s.ckmask[q * KMAX * B + lane] = s.kmask[warp * KMAX * B + lane];
            __syncwarp();
            if (lane == 0) {
                cm[1] = ctl.kcnt[warp];
                cm[0] = ctl.epoch;
            }
        }
        // Leading run of deterministic measurements, resets included: a
        // reset's X only flips signs (rows < 2n keep their x and z), so the
        // later measurements of the run stay deterministic with the same rows;
        // their outcomes are corrected for the earlier resets below.  Read
        // the status words before the next barrier: the next window's scan
        // overwrites them.
        int P = 0;
        while (P < act && ctl.status[P] != ST_OTHER) ++P;
        if (tid < NW) ctl.resq[tid] = (tid < P && ctl.status[tid] == ST_DET_RESET) ? ctl.wop[tid].q : -1;
        __syncthreads();
        bool any_reset = false;
        for (int j = 0; j < P; ++j) any_reset |= ctl.resq[j] >= 0;
        if (warp < P) {
            warp_det<B>(X, Z, R, n, w, k0, s.klist + warp * KMAX, s.kmask + warp * KMAX * B, ctl.kcnt[warp],
                        warp == P - 1, warp, ctl.resq, s.wraw, s.wz);
            const MeasOp &op = ctl.wop[warp];
            if (op.kstat && k0 == 0 && (tid & 31) == 0) {
                op.kstat[0] = 0;
                op.kstat[1] = ctl.kcnt[warp];
            }
        }
        __syncthreads();
        if (P > 0) {
            // Outcomes in order: measurement j sees the X of every earlier
            // reset r of the run on the shots where r's outcome is 1 (a chain
            // through shared memory, only when the run holds a reset).
            if (any_reset) {
                if (tid < B) {
                    const int b = tid;
                    for (int j = 0; j < P; ++j) {
                        u64 v = s.wraw[j * B + b];
                        for (int r = 0; r < j; ++r)
                            if (ctl.resq[r] >= 0) v ^= s.wres[r * B + b] & s.wz[(j * NW + r) * B + b];
                        s.wres[j * B + b] = v;
                    }
                }
                __syncthreads();
            }
            const u64 *fin = any_reset ? s.wres : s.wraw;
            for (int e = tid; e < P * B; e += blockDim.x) {
                const int j = e / B, b = e % B;
                const MeasOp &op = ctl.wop[j];
                op.res[k0 + b] = fin[j * B + b];
                op.det[k0 + b] = ~0ull;
                if (j == P - 1) R[2 * n * w + k0 + b] = fin[j * B + b];  // the scratch row the last one left
            }
            __syncthreads();
            if (any_reset) {
                // Every reset's X on rows 0..2n-1; the scratch row only sees
                // the last measurement's own reset (later measurements
                // rewrite it).
                const int64_t Wr = 2 * n + 1;
                for (int64_t e = tid; e < Wr * B; e += blockDim.x) {
                    const int64_t i = e / B;
                    const int b = (int)(e % B);
                    const int64_t k = k0 + b;
                    u64 acc = 0ull;
                    if (i < 2 * n) {
                        for (int r = 0; r < P; ++r)
                            if (ctl.resq[r] >= 0) acc ^= fin[r * B + b] & Z[(i * n + ctl.resq[r]) * w + k];
                    } else if (ctl.resq[P - 1] >= 0) {
                        acc = fin[(P - 1) * B + b] & Z[(i * n + ctl.resq[P - 1]) * w + k];
                    }
                    if (acc) R[i * w + k] ^= acc;
                }
                __syncthreads();
            }
        }
        pos += P;
        if (P < act) {
            const MeasOp op = ops[pos];
            if (use_cache && tid == 0) ctl.epoch++;  // rows may change: every cached scan is stale
            cta_measure<B>(X, Z, R, n, w, k0, op, s, ctl, seed, event_base, word_base);
            if (op.reset) cta_reset_flip<B>(Z, R, n, w, k0, op);
            pos += 1;
            window = 2;
        } else {
            window = min(NW, window * 2);
        }
    }
}

size_t smem_bytes(int64_t n, int B, bool cache = false) {
    return (size_t)(2 * n * B + 2 * n * B + STEP_CHUNK * NW * 2 + NW * KMAX * B + 2 * NW * B + NW * NW * B +
                    (cache ? n * KMAX * B : 0)) *
               sizeof(u64) +
           (size_t)(2 * n + NW * KMAX + (cache ? n * (2 + KMAX) : 0)) * sizeof(int);
}

template <int B>
int launch_b(cudaStream_t stream, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, const MeasOp *dev_ops, int nops,
             uint64_t seed, uint64_t word_base, const RunParams *rp, int window) {
    // The scan cache when the window path runs and it fits.
    const int cache = window > 0 && smem_bytes(n, B, true) <= kMeasSmemMax ? 1 : 0;
    const size_t smem = smem_bytes(n, B, cache != 0);
    if (smem + sizeof(Ctl) > 48 * 1024) {  // static and dynamic shared memory share the default limit
        const int rc = allow_max_smem((const void *)measure_kernel<B>);
        if (rc != OK) return rc;
    }
    measure_kernel<B><<<(unsigned)(w / B), NW * 32, smem, stream>>>(X, Z, R, n, w, dev_ops, nops, seed, word_base, rp,
                                                                    window, cache);
    PS_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace

int measure_words_per_cta(int64_t n, int64_t w) {
    for (int B = 2; B > 1; B >>= 1)
        if (w % B == 0 && smem_bytes(n, B) <= 200 * 1024 && w / B >= 1) return B;
    return 1;
}

int launch_measure_list(cudaStream_t stream, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, const MeasOp *dev_ops,
                        int nops, uint64_t seed, uint64_t word_base, const RunParams *rp, int words_per_cta) {
    if (nops <= 0) return OK;
    if (n > (int64_t)NW * 32 * MAXC) return fail(E_ARG, "too many qubits for the measurement kernel (max 2048)");
    // A single measurement has no window to overlap: spread it over the most
    // CTAs (one word each).
    int B = nops == 1 ? 1 : measure_words_per_cta(n, w);
    if (nops > 1 && words_per_cta == 1) B = 1;
    if (nops > 1 && words_per_cta == 2 && w % 2 == 0 && smem_bytes(n, 2) <= kMeasSmemMax) B = 2;
    if (nops > 1 && words_per_cta == 4 && w % 4 == 0 && smem_bytes(n, 4) <= kMeasSmemMax) B = 4;
    if (smem_bytes(n, B) > kMeasSmemMax) return fail(E_ARG, "measurement tile does not fit in shared memory");
    const int window = nops == 1 ? 0 : NW;
    if (B == 4) return launch_b<4>(stream, X, Z, R, n, w, dev_ops, nops, seed, word_base, rp, window);
    if (B == 2) return launch_b<2>(stream, X, Z, R, n, w, dev_ops, nops, seed, word_base, rp, window);
    return launch_b<1>(stream, X, Z, R, n, w, dev_ops, nops, seed, word_base, rp, window);
}

int launch_measure(ps_state *h, const MeasOp *ops_host, int nops) {
    if ((size_t)nops > h->meas_cap) {
        // A pooled buffer is reused as soon as it is returned: let the
        // launches that read the old one finish first.
        if (h->pool && h->meas_buf) PS_CUDA(cudaStreamSynchronize(h->stream));
        dev_free(h, h->meas_buf);
        h->meas_buf = nullptr;
        h->meas_cap = 0;
        void *p = nullptr;
        if (dev_alloc(h, &p, (size_t)nops * sizeof(MeasOp)) != OK) return E_NOMEM;
        h->meas_buf = (MeasOp *)p;
        h->meas_cap = (size_t)nops;
    }
    PS_CUDA(cudaMemcpyAsync(h->meas_buf, ops_host, (size_t)nops * sizeof(MeasOp), cudaMemcpyHostToDevice, h->stream));
    return launch_measure_list(h->stream, h->X, h->Z, h->R, h->n, h->w, h->meas_buf, nops, (uint64_t)h->seed,
                               (uint64_t)h->word_base,
                               nullptr);
}

}  // namespace ps
