// ps_measure.cu -- Z-basis measurement (Aaronson-Gottesman), 64 shots per
// CTA, bit-exact with the reference's BatchMeasureFunctor
// (MeasurementFunctors.hpp:267-318).
//
// One CTA owns one 64-shot word and runs a list of measurements in order.
// Per measurement of qubit q:
//  1. the x bits of column q for rows 0..2n-1 are staged in shared memory;
//  2. warp 0 finds, per shot, the lowest stabilizer row p+n with x(p+n,q)=1
//     (ballot + ffs, :297-301).  Shots sharing a pivot p form a group; shots
//     with none take the deterministic branch;
//  3. random branch per group (MeasureRandom, :225-265): row p+n is copied
//     to row p, row p+n becomes +-Z_q with the drawn outcome, then every row
//     i != p, p+n with x(i,q)=1 is multiplied by the copied row.  Those
//     row multiplications are independent: one warp per row, lanes over
//     columns, and the mod-4 phase sum (RowProductSign, :97-129) is a
//     bit-sliced 2-bit counter per shot reduced with warp shuffles;
//  4. deterministic branch (MeasureDetermined, :189-201): the scratch row
//     accumulates the stabilizer rows i+n with x(i,q)=1 in increasing i.
//     Each thread owns a set of columns and keeps their running product in
//     registers; the phase sum of every step is reduced separately, so the
//     reference's per-step rounding (bit 1 of each step's sum) is kept exactly
//     even for tableaux whose rows do not commute.
#include <vector>

#include "ps_internal.h"
#include "ps_segment.cuh"

namespace ps {

namespace {

constexpr int MAXC = 8;        // columns per thread in the deterministic branch
constexpr int STEP_CHUNK = 32;  // deterministic steps reduced per round

struct MeasSmem {
    u64 outcome;
    u64 racc;
    int ngroups;
    int cnt;
    u64 det_mask;
    int gp[64];
    u64 gm[64];
    u64 pr;
};

__device__ __forceinline__ void warp_phase_reduce(u64 &c1, u64 &c0) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const u64 d1 = __shfl_xor_sync(0xffffffffu, c1, off);
        const u64 d0 = __shfl_xor_sync(0xffffffffu, c0, off);
        phase_add(c1, c0, d1, d0);
    }
}

__global__ void __launch_bounds__(1024) measure_kernel(u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w,
                                                      const MeasOp *__restrict__ ops, int nops, uint64_t seed_arg,
                                                      uint64_t word_base, const RunParams *__restrict__ rp) {
    const uint64_t seed = rp ? rp->seed : seed_arg;
    const uint64_t event_base = rp ? rp->event_base : 0ull;
    extern __shared__ u64 dyn[];
    __shared__ MeasSmem sm;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = T >> 5;
    const int64_t k = blockIdx.x;
    const int64_t W = 2 * n + 1;
    u64 *col = dyn;                                  // 2n
    u64 *prow_x = col + 2 * n;                       // n
    u64 *prow_z = prow_x + n;                        // n
    u64 *part = prow_z + n;                          // STEP_CHUNK * nwarps * 2
    int *rowlist = reinterpret_cast<int *>(part + STEP_CHUNK * nwarps * 2);  // 2n

    for (int oi = 0; oi < nops; ++oi) {
        const MeasOp op = ops[oi];
        const int64_t q = op.q;
        // 1. column q of rows 0..2n-1
        for (int64_t i = tid; i < 2 * n; i += T) col[i] = X[(i * n + q) * w + k];
        __syncthreads();
        // 2. pivot groups
        if (warp == 0) {
            u64 rem = ~0ull;
            int ng = 0;
            int64_t p0 = 0;
            while (rem && p0 < n) {
                bool found = false;
                for (int64_t base = p0; base < n; base += 32) {
                    const int64_t p = base + lane;
                    const u64 v = (p < n) ? (col[n + p] & rem) : 0ull;
                    const unsigned bal = __ballot_sync(0xffffffffu, v != 0ull);
                    if (bal) {
                        const int f = __ffs(bal) - 1;
                        const u64 hit = __shfl_sync(0xffffffffu, v, f);
                        if (lane == 0) {
                            sm.gp[ng] = (int)(base + f);
                            sm.gm[ng] = hit;
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
            if (lane == 0) {
                sm.ngroups = ng;
                sm.det_mask = rem;
                sm.racc = 0ull;
            }
            // Outcome draws for the random branch (all 64 shots; only
            // group members use them).
            if (ng > 0) {
                u64 bits = 0ull;
                if (lane < 16) {
                    if (op.forced) {
                        const u64 fw = op.forced[k];
#pragma unroll
                        for (int l = 0; l < 4; ++l) {
                            const int b = lane * 4 + l;
                            const float u = ((fw >> b) & 1ull) ? 0.25f : 0.75f;
                            if (u < op.bias) bits |= 1ull << b;
                        }
                    } else {
                        const u32x4 u = draw_block(seed, event_base + op.event, word_base + (uint64_t)k, (uint32_t)lane, TAG_MEASURE);
#pragma unroll
                        for (int l = 0; l < 4; ++l)
                            if (unit_float(u.v[l]) < op.bias) bits |= 1ull << (lane * 4 + l);
                    }
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) bits |= __shfl_xor_sync(0xffffffffu, bits, off);
                if (lane == 0) sm.outcome = bits;
            }
        }
        __syncthreads();
        const int ng = sm.ngroups;
        const u64 outcome = sm.outcome;
        u64 res_word = 0ull;
        int rows_done = 0;
        // 3. random branch, one group of shots (same pivot) at a time
        for (int g = 0; g < ng; ++g) {
            const int64_t p = sm.gp[g];
            const u64 m = sm.gm[g];
            for (int64_t j = tid; j < n; j += T) {
                prow_x[j] = X[((p + n) * n + j) * w + k];
                prow_z[j] = Z[((p + n) * n + j) * w + k];
            }
            if (tid == 0) {
                sm.pr = R[(p + n) * w + k];
                sm.cnt = 0;
            }
            __syncthreads();
            const u64 pr = sm.pr;
            // CopyFromRowAtoRowB(p+n -> p) and ZeroRow(p+n); z(p+n,q) = 1.
            for (int64_t j = tid; j < n; j += T) {
                const int64_t o = (p * n + j) * w + k, o2 = ((p + n) * n + j) * w + k;
                X[o] = (X[o] & ~m) | (prow_x[j] & m);
                Z[o] = (Z[o] & ~m) | (prow_z[j] & m);
                X[o2] &= ~m;
                Z[o2] = (Z[o2] & ~m) | (j == q ? m : 0ull);
            }
            if (tid == 0) {
                R[p * w + k] = (R[p * w + k] & ~m) | (pr & m);
                R[(p + n) * w + k] = (R[(p + n) * w + k] & ~m) | (outcome & m);
            }
            for (int64_t i = tid; i < 2 * n; i += T)
                if (i != p && i != p + n && (col[i] & m)) rowlist[atomicAdd(&sm.cnt, 1)] = (int)i;
            __syncthreads();
            const int cnt = sm.cnt;
            rows_done += cnt;
            for (int t = warp; t < cnt; t += nwarps) {
                const int64_t i = rowlist[t];
                const u64 mi = col[i] & m;
                u64 c1 = 0ull, c0 = 0ull;
                for (int64_t j = lane; j < n; j += 32) {
                    const int64_t o = (i * n + j) * w + k;
                    const u64 xi = X[o], zi = Z[o], xp = prow_x[j], zp = prow_z[j];
                    phase_accumulate(xi, zi, xp, zp, mi, c1, c0);
                    X[o] = xi ^ (xp & mi);
                    Z[o] = zi ^ (zp & mi);
                }
                warp_phase_reduce(c1, c0);
                if (lane == 0) {
                    const u64 ri = R[i * w + k];
                    R[i * w + k] = (ri & ~mi) | ((ri ^ pr ^ c1) & mi);
                }
            }
            res_word |= outcome & m;
            __syncthreads();
        }
        // 4. deterministic branch
        const u64 dm = sm.det_mask;
        if (dm) {
            if (warp == 0) {
                int cnt = 0;
                for (int64_t base = 0; base < n; base += 32) {
                    const int64_t i = base + lane;
                    const bool v = i < n && (col[i] & dm);
                    const unsigned bal = __ballot_sync(0xffffffffu, v);
                    if (v) rowlist[cnt + __popc(bal & ((1u << lane) - 1u))] = (int)i;
                    cnt += __popc(bal);
                }
                if (lane == 0) sm.cnt = cnt;
            }
            __syncthreads();
            const int cnt = sm.cnt;
            rows_done += cnt;
            u64 ax[MAXC], az[MAXC];
#pragma unroll
            for (int u = 0; u < MAXC; ++u) ax[u] = az[u] = 0ull;
            for (int c0s = 0; c0s < cnt; c0s += STEP_CHUNK) {
                const int len = min(STEP_CHUNK, cnt - c0s);
                for (int t = 0; t < len; ++t) {
                    const int64_t i = rowlist[c0s + t];
                    const u64 mt = col[i] & dm;
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
                    warp_phase_reduce(c1, c0);
                    if (lane == 0) {
                        part[(t * nwarps + warp) * 2] = c1;
                        part[(t * nwarps + warp) * 2 + 1] = c0;
                    }
                }
                __syncthreads();
                if (tid < len) {
                    const int t = tid;
                    u64 s1 = 0ull, s0 = 0ull;
                    for (int wv = 0; wv < nwarps; ++wv) phase_add(s1, s0, part[(t * nwarps + wv) * 2], part[(t * nwarps + wv) * 2 + 1]);
                    const int64_t i = rowlist[c0s + t];
                    const u64 mt = col[i] & dm;
                    const u64 contrib = (R[(i + n) * w + k] ^ s1) & mt;
                    atomicXor(&sm.racc, contrib);
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
            const u64 racc = sm.racc;
            if (tid == 0) R[srow * w + k] = (R[srow * w + k] & ~dm) | racc;
            res_word |= racc & dm;
        }
        if (tid == 0) {
            op.res[k] = res_word;
            op.det[k] = dm;
            if (op.kstat && k == 0) {
                op.kstat[0] = ng > 0;
                op.kstat[1] = rows_done;
            }
        }
        __syncthreads();
        // ResetQubit: X on shots with outcome 1 flips rows with Z on q.
        if (op.reset)
            for (int64_t i = tid; i < W; i += T) R[i * w + k] ^= res_word & Z[(i * n + q) * w + k];
        __syncthreads();
    }
}

}  // namespace

size_t measure_smem_bytes(int64_t n, int threads) {
    return (size_t)(4 * n + STEP_CHUNK * (threads / 32) * 2) * sizeof(u64) + (size_t)2 * n * sizeof(int);
}

int measure_threads(int64_t n) { return n <= 256 * MAXC ? 256 : 1024; }

int launch_measure_list(cudaStream_t stream, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, const MeasOp *dev_ops,
                        int nops, uint64_t seed, uint64_t word_base, const RunParams *rp) {
    const int T = measure_threads(n);
    if (n > (int64_t)T * MAXC) return fail(E_ARG, "too many qubits for the measurement kernel (max 8192)");
    const size_t smem = measure_smem_bytes(n, T);
    if (smem > 48 * 1024)
        PS_CUDA(cudaFuncSetAttribute(measure_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    measure_kernel<<<(unsigned)w, T, smem, stream>>>(X, Z, R, n, w, dev_ops, nops, seed, word_base, rp);
    PS_CUDA(cudaGetLastError());
    return OK;
}

int launch_measure(ps_state *h, const MeasOp *ops_host, int nops) {
    if ((size_t)nops > h->meas_cap) {
        cudaFree(h->meas_buf);
        h->meas_buf = nullptr;
        h->meas_cap = 0;
        PS_CUDA(cudaMalloc(&h->meas_buf, (size_t)nops * sizeof(MeasOp)));
        h->meas_cap = (size_t)nops;
    }
    PS_CUDA(cudaMemcpyAsync(h->meas_buf, ops_host, (size_t)nops * sizeof(MeasOp), cudaMemcpyHostToDevice, h->stream));
    return launch_measure_list(h->stream, h->X, h->Z, h->R, h->n, h->w, h->meas_buf, nops, (uint64_t)h->seed, 0, nullptr);
}

}  // namespace ps
