// ps_segment.cu -- the fused form of a run of gates ("segment"): every gate,
// Pauli gate, Pauli channel and reset-X between two measurement phases is
// applied in ONE pass over the tableau.
//
// A CTA stages a tile -- ROWS tableau rows x BW shot-words x the segment's
// touched columns -- from HBM into shared memory (transposed so that the
// columns of one (row, word) are contiguous), applies the whole gate
// schedule there, and writes the tile back once.  One warp owns one
// (row, word) pair: it walks the layers (gates within a layer act on
// disjoint columns, so lanes take different gates), accumulates its r
// updates in a register (gates and sign ops only ever XOR into r) and
// reduces them once at the end.  HBM traffic per segment is therefore the
// touched x/z columns and r read and written once: 2 * (2|Q|+1) * W * S/8
// bytes.
#include <algorithm>

#include "ps_internal.h"
#include "ps_segment.cuh"

namespace ps {

namespace {

// Pauli-channel sampling for one segment, pass 1: 16 threads per (word,
// channel); thread `sub` draws Philox block `sub` (shots 4*sub..4*sub+3 of
// the word) and the X/Z component masks are OR-reduced over the 16 lanes into
// dense[word][slot].
__global__ void __launch_bounds__(256) noise_dense_kernel(SegmentDev seg, int64_t w, const RunParams *__restrict__ rp) {
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t pair = gt >> 4;
    const uint32_t sub = (uint32_t)(gt & 15);
    const int64_t k = pair / seg.nslots;
    const int s = (int)(pair - k * seg.nslots);
    u64 fxa = 0, fza = 0, fxb = 0, fzb = 0;
    if (k < w) {
        const NoiseSlot sl = seg.slots[s];
        const uint64_t *thr = seg.thr + sl.thr_off;
        const uint64_t total = thr[sl.count - 1];
        const u32x4 u = draw_block(rp->seed, rp->event_base + sl.event, (uint64_t)k, sub, TAG_NOISE);
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const uint64_t v = u.v[l];
            if (v >= total) continue;  // identity, the common case
            int idx = 1;
            while (v >= thr[idx - 1]) ++idx;
            const u64 bit = 1ull << (sub * 4 + l);
            const int pa = sl.count == 3 ? idx : (idx >> 2), pb = sl.count == 3 ? 0 : (idx & 3);
            if (pa == 1 || pa == 2) fxa |= bit;
            if (pa == 2 || pa == 3) fza |= bit;
            if (pb == 1 || pb == 2) fxb |= bit;
            if (pb == 2 || pb == 3) fzb |= bit;
        }
    }
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) {
        fxa |= __shfl_xor_sync(0xffffffffu, fxa, off);
        fza |= __shfl_xor_sync(0xffffffffu, fza, off);
        fxb |= __shfl_xor_sync(0xffffffffu, fxb, off);
        fzb |= __shfl_xor_sync(0xffffffffu, fzb, off);
    }
    if (sub == 0 && k < w) {
        u64 *d = seg.dense + pair * 4;
        d[0] = fxa;
        d[1] = fza;
        d[2] = fxb;
        d[3] = fzb;
    }
}

// Pass 2: one warp per word appends the non-identity outcomes to the word's
// entry list; ballot compaction keeps slot (= layer) order.
__global__ void __launch_bounds__(128) noise_compact_kernel(SegmentDev seg, int64_t w) {
    const int lane = threadIdx.x & 31;
    const int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= w) return;
    int count = 0;
    NoiseEntry *out = seg.entries + k * (int64_t)seg.cap;
    const u64 *dense = seg.dense + k * (int64_t)seg.nslots * 4;
    for (int base = 0; base < seg.nslots; base += 32) {
        const int s = base + lane;
        u64 fxa = 0, fza = 0, fxb = 0, fzb = 0;
        if (s < seg.nslots) {
            const ulonglong2 a = *reinterpret_cast<const ulonglong2 *>(dense + (int64_t)s * 4);
            const ulonglong2 b = *reinterpret_cast<const ulonglong2 *>(dense + (int64_t)s * 4 + 2);
            fxa = a.x;
            fza = a.y;
            fxb = b.x;
            fzb = b.y;
        }
        const bool hit = (fxa | fza | fxb | fzb) != 0ull;
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (hit) {
            const int pos = count + __popc(bal & ((1u << lane) - 1u));
            const NoiseSlot sl = seg.slots[s];
            NoiseEntry e;
            e.fxa = fxa;
            e.fza = fza;
            e.fxb = fxb;
            e.fzb = fzb;
            e.layer = sl.layer;
            e.a = (uint16_t)sl.a;
            e.b = sl.b >= 0 ? (uint16_t)sl.b : (uint16_t)0xFFFF;
            out[pos] = e;
        }
        count += __popc(bal);
    }
    if (lane == 0) seg.entry_count[k] = count;
}

// Tile cell: x and z of one (row, word, column) side by side, so a gate
// reads / writes a column with one 16-byte shared-memory access.
typedef ulonglong2 XZ;

__device__ __forceinline__ void apply_gate(const SegGate g, XZ *__restrict__ t, u64 &rd,
                                           const u64 *const *__restrict__ recs, int64_t kg) {
    const int a = g.a;
    switch (g.code_rec & 15) {
    case OP_H: {  // GateFunctors.hpp:90-93
        const XZ v = t[a];
        rd ^= v.x & v.y;
        t[a] = make_ulonglong2(v.y, v.x);
        break;
    }
    case OP_S: {  // :165-169
        const XZ v = t[a];
        rd ^= v.x & v.y;
        t[a] = make_ulonglong2(v.x, v.y ^ v.x);
        break;
    }
    case OP_CX: {  // :248-253
        const XZ c = t[a], u = t[g.b];
        rd ^= c.x & u.y & ~(u.x ^ c.y);
        t[g.b] = make_ulonglong2(u.x ^ c.x, u.y);
        t[a] = make_ulonglong2(c.x, c.y ^ u.y);
        break;
    }
    case OP_CZ: {  // :30-35
        const XZ c = t[a], u = t[g.b];
        rd ^= c.x & u.x & (u.y ^ c.y);
        t[g.b] = make_ulonglong2(u.x, u.y ^ c.x);
        t[a] = make_ulonglong2(c.x, c.y ^ u.x);
        break;
    }
    case OP_H_IF: {  // :143-148
        const u64 f = recs[g.code_rec >> 4][kg];
        const XZ v = t[a];
        rd ^= f & v.x & v.y;
        t[a] = make_ulonglong2((v.x & ~f) | (v.y & f), (v.y & ~f) | (v.x & f));
        break;
    }
    case OP_S_IF: {  // :221-228
        const u64 f = recs[g.code_rec >> 4][kg];
        const XZ v = t[a];
        rd ^= f & v.x & v.y;
        t[a] = make_ulonglong2(v.x, v.y ^ (f & v.x));
        break;
    }
    default: break;
    }
}

// A layer whose gates all have one code: the branch is taken once per layer
// and every lane keeps two independent gates in flight.
template <int CODE>
__device__ __forceinline__ void layer_uniform(const SegGate *__restrict__ gates, int g0, int g1, int lane,
                                              XZ *__restrict__ t, u64 &rd) {
    for (int g = g0 + lane; g < g1; g += 64) {
        const bool two = g + 32 < g1;
        const SegGate ga = gates[g];
        const SegGate gb = two ? gates[g + 32] : ga;
        if (CODE == OP_H || CODE == OP_S) {
            const XZ va = t[ga.a];
            const XZ vb = t[gb.a];
            rd ^= va.x & va.y;
            t[ga.a] = CODE == OP_H ? make_ulonglong2(va.y, va.x) : make_ulonglong2(va.x, va.y ^ va.x);
            if (two) {
                rd ^= vb.x & vb.y;
                t[gb.a] = CODE == OP_H ? make_ulonglong2(vb.y, vb.x) : make_ulonglong2(vb.x, vb.y ^ vb.x);
            }
        } else {
            const XZ ca = t[ga.a], ua = t[ga.b];
            const XZ cb = t[gb.a], ub = t[gb.b];
            if (CODE == OP_CX) {
                rd ^= ca.x & ua.y & ~(ua.x ^ ca.y);
                t[ga.b] = make_ulonglong2(ua.x ^ ca.x, ua.y);
                t[ga.a] = make_ulonglong2(ca.x, ca.y ^ ua.y);
                if (two) {
                    rd ^= cb.x & ub.y & ~(ub.x ^ cb.y);
                    t[gb.b] = make_ulonglong2(ub.x ^ cb.x, ub.y);
                    t[gb.a] = make_ulonglong2(cb.x, cb.y ^ ub.y);
                }
            } else {
                rd ^= ca.x & ua.x & (ua.y ^ ca.y);
                t[ga.b] = make_ulonglong2(ua.x, ua.y ^ ca.x);
                t[ga.a] = make_ulonglong2(ca.x, ca.y ^ ua.x);
                if (two) {
                    rd ^= cb.x & ub.x & (ub.y ^ cb.y);
                    t[gb.b] = make_ulonglong2(ub.x, ub.y ^ cb.x);
                    t[gb.a] = make_ulonglong2(cb.x, cb.y ^ ub.x);
                }
            }
        }
    }
}

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ void apply_entry(const NoiseEntry &en, const XZ *__restrict__ t, u64 &rd) {
    const XZ va = t[en.a];
    rd ^= (en.fxa & va.y) ^ (en.fza & va.x);
    if (en.b != 0xFFFF) {
        const XZ vb = t[en.b];
        rd ^= (en.fxb & vb.y) ^ (en.fzb & vb.x);
    }
}

constexpr int NE = 3;  // channel outcomes a lane keeps in registers (32*NE per word)

// Persistent: each CTA stages the segment's schedule and column map in shared
// memory once, then loops over tiles (ROWS rows x BW words x nq columns).
// Tile cells are copied with 8-byte cp.async straight into their slots (all
// copies of a tile in flight at once), processed, and stored back.
__global__ void __launch_bounds__(256, 3) segment_kernel(u64 *__restrict__ X, u64 *__restrict__ Z,
                                                        u64 *__restrict__ R, int64_t n, int64_t W, int64_t w,
                                                        SegmentDev seg, int rows, int bw, int64_t nchunks,
                                                        int64_t ntiles, const u64 *const *__restrict__ recs) {
    extern __shared__ u64 sm[];
    const int nq = seg.nq;
    const int T = blockDim.x, tid = threadIdx.x;
    // Tile row: nq columns + a zero dummy column, padded to an odd number of
    // 16-byte cells so the 8 words of one column fall on distinct bank groups.
    const int nq1 = (nq + 1) | 1;
    SegLayer *s_layers = reinterpret_cast<SegLayer *>(sm);
    SegRun *s_runs = reinterpret_cast<SegRun *>(s_layers + seg.nlayers);
    SegGate *s_gates = reinterpret_cast<SegGate *>(s_runs + seg.nruns);
    SegSign *s_signs = reinterpret_cast<SegSign *>(s_gates + seg.ngates);
    int32_t *s_cols = reinterpret_cast<int32_t *>(s_signs + seg.nsigns);
    const size_t head = ((size_t)seg.nlayers * sizeof(SegLayer) + (size_t)seg.nruns * sizeof(SegRun) +
                         (size_t)seg.ngates * sizeof(SegGate) + (size_t)seg.nsigns * sizeof(SegSign) +
                         (size_t)nq * sizeof(int32_t) + 15) / 16 * 2;
    const u64 **s_recp = reinterpret_cast<const u64 **>(sm + head);  // [nrecsig] record pointers
    XZ *tile_xz = reinterpret_cast<XZ *>(sm + head + (seg.nrecsig + 1) / 2 * 2);  // [rows*bw][nq1]
    u64 *rtile = reinterpret_cast<u64 *>(tile_xz + (size_t)rows * bw * nq1);      // [rows*bw] r words
    u64 *s_recw = rtile + rows * bw;                                               // [bw][nrecsig]
    for (int i = tid; i < seg.nrecsig; i += T) s_recp[i] = recs[seg.recsig_rec[i]];
    for (int i = tid; i < seg.nlayers; i += T) s_layers[i] = seg.layers[i];
    for (int i = tid; i < seg.nruns; i += T) s_runs[i] = seg.runs[i];
    for (int i = tid; i < seg.ngates; i += T) s_gates[i] = seg.gates[i];
    for (int i = tid; i < seg.nsigns; i += T) s_signs[i] = seg.signs[i];
    for (int i = tid; i < nq; i += T) s_cols[i] = seg.cols[i];
    __syncthreads();

    const int lane = tid & 31, wid = tid >> 5, nw = T >> 5;
    // Load / store mapping: lane -> word kk_t = lane % bw and column slot
    // jj = lane / bw; one warp instruction covers columns cb + c + 8*jj, which
    // keeps the 8-byte shared-memory writes of a half-warp on distinct banks.
    const int kk_t = lane % bw, jj = lane / bw, jn = 32 / bw;
    const int span = 8 * jn;  // columns one warp covers in 8 instructions
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t row0 = (tile / nchunks) * rows;
        const int64_t k0 = (tile % nchunks) * bw;
        // ---- load
        for (int r = 0; r < rows; ++r) {
            const int64_t row = row0 + r;
            const int64_t kg = k0 + kk_t;
            const bool ok = row < W && kg < w;
            XZ *d = tile_xz + (size_t)(r * bw + kk_t) * nq1;
            const int64_t rbase = row * n * w + kg;
            if (tid < bw) d[nq] = make_ulonglong2(0ull, 0ull);
            for (int cb = wid * span; cb < nq; cb += nw * span)
                for (int c = 0; c < 8; ++c) {
                    const int l = cb + c + 8 * jj;
                    if (l >= nq) continue;
                    if (ok) {
                        const int64_t off = rbase + (int64_t)s_cols[l] * w;
                        cp_async8(&d[l].x, X + off);
                        cp_async8(&d[l].y, Z + off);
                    } else {
                        d[l] = make_ulonglong2(0ull, 0ull);
                    }
                }
        }
        for (int pair = tid; pair < rows * bw; pair += T) {
            const int64_t row = row0 + pair / bw, kg = k0 + pair % bw;
            if (row < W && kg < w) cp_async8(&rtile[pair], R + row * w + kg);
        }
        for (int e = tid; e < seg.nrecsig * bw; e += T) {
            const int kk = e % bw, slot = e / bw;
            const int64_t kg = k0 + kk;
            if (kg < w) cp_async8(&s_recw[kk * seg.nrecsig + slot], s_recp[slot] + kg);
        }
        cp_async_wait_all();
        __syncthreads();

        // ---- apply the schedule: warp = (row, word)
        for (int pair = wid; pair < rows * bw; pair += nw) {
            const int r = pair / bw, kk = pair % bw;
            const int64_t row = row0 + r, kg = k0 + kk;
            u64 rd = 0ull;
            if (row < W && kg < w) {
                XZ *t = tile_xz + (size_t)pair * nq1;
                const NoiseEntry *ent = seg.entries ? seg.entries + kg * (int64_t)seg.cap : nullptr;
                const int nent = seg.entries ? seg.entry_count[kg] : 0;
                NoiseEntry mine[NE];
#pragma unroll
                for (int u = 0; u < NE; ++u) {
                    const int e = lane + 32 * u;
                    if (e < nent) {
                        mine[u] = ent[e];
                    } else {
                        mine[u].layer = -1;
                    }
                }
                const bool spill = nent > 32 * NE;
                int cursor = 32 * NE;
                for (int L = 0; L < seg.nlayers; ++L) {
                    const SegLayer ly = s_layers[L];
                    for (int ri = ly.r0; ri < ly.r1; ++ri) {  // runs touch disjoint columns
                        const SegRun rn = s_runs[ri];
                        switch (rn.code) {
                        case OP_H: layer_uniform<OP_H>(s_gates, rn.g0, rn.g1, lane, t, rd); break;
                        case OP_S: layer_uniform<OP_S>(s_gates, rn.g0, rn.g1, lane, t, rd); break;
                        case OP_CX: layer_uniform<OP_CX>(s_gates, rn.g0, rn.g1, lane, t, rd); break;
                        case OP_CZ: layer_uniform<OP_CZ>(s_gates, rn.g0, rn.g1, lane, t, rd); break;
                        default:
                            for (int g = rn.g0 + lane; g < rn.g1; g += 32) apply_gate(s_gates[g], t, rd, recs, kg);
                        }
                    }
                    __syncwarp();
                    for (int s = ly.s0 + lane; s < ly.s1; s += 32) {
                        const SegSign sg = s_signs[s];
                        const XZ v = t[sg.a];
                        if (sg.kind == SIGN_X)
                            rd ^= v.y;
                        else if (sg.kind == SIGN_Y)
                            rd ^= v.x ^ v.y;
                        else if (sg.kind == SIGN_Z)
                            rd ^= v.x;
                        else
                            rd ^= s_recw[kk * seg.nrecsig + sg.rec] & v.y;
                    }
#pragma unroll
                    for (int u = 0; u < NE; ++u)
                        if (mine[u].layer == L) apply_entry(mine[u], t, rd);
                    if (spill) {  // more outcomes than the registers hold
                        while (cursor < nent) {
                            const int e = cursor + lane;
                            const bool take = e < nent && ent[e].layer == L;
                            const unsigned bal = __ballot_sync(0xffffffffu, take);
                            if (take) {
                                const NoiseEntry en = ent[e];
                                apply_entry(en, t, rd);
                            }
                            const int c = __popc(bal);
                            cursor += c;
                            if (c < 32) break;
                        }
                    }
                    __syncwarp();
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) rd ^= __shfl_xor_sync(0xffffffffu, rd, off);
            if (lane == 0) rtile[pair] ^= rd;
        }
        __syncthreads();

        // ---- store back
        for (int r = 0; r < rows; ++r) {
            const int64_t row = row0 + r;
            const int64_t kg = k0 + kk_t;
            if (!(row < W && kg < w)) continue;
            const XZ *d = tile_xz + (size_t)(r * bw + kk_t) * nq1;
            const int64_t rbase = row * n * w + kg;
            for (int cb = wid * span; cb < nq; cb += nw * span)
                for (int c = 0; c < 8; ++c) {
                    const int l = cb + c + 8 * jj;
                    if (l >= nq) continue;
                    const int64_t off = rbase + (int64_t)s_cols[l] * w;
                    const XZ v = d[l];
                    X[off] = v.x;
                    Z[off] = v.y;
                }
        }
        for (int pair = tid; pair < rows * bw; pair += T) {
            const int64_t row = row0 + pair / bw, kg = k0 + pair % bw;
            if (row < W && kg < w) R[row * w + kg] = rtile[pair];
        }
        __syncthreads();
    }
}

int g_num_sms = 0;

}  // namespace

size_t segment_smem_bytes(int nq, int rows, int bw) { return (size_t)rows * bw * (2 * ((size_t)(nq + 1) | 1) + 1) * sizeof(u64); }

size_t segment_launch_smem(int nlayers, int nruns, int ngates, int nsigns, int nq, int nrecsig, int rows, int bw) {
    const size_t sched = ((size_t)nlayers * sizeof(SegLayer) + (size_t)nruns * sizeof(SegRun) +
                          (size_t)ngates * sizeof(SegGate) + (size_t)nsigns * sizeof(SegSign) +
                          (size_t)nq * sizeof(int32_t) + 15) / 16 * 16 +
                         (size_t)(nrecsig + 1) / 2 * 16 + (size_t)nrecsig * bw * 8 + (size_t)rows * bw * 8;
    return segment_smem_bytes(nq, rows, bw) + sched;
}

int launch_noise_sample(cudaStream_t stream, const SegmentDev &seg, int64_t w, const RunParams *rp) {
    if (seg.nslots == 0) return OK;
    const int64_t threads = 16 * (int64_t)seg.nslots * w;
    noise_dense_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, stream>>>(seg, w, rp);
    PS_CUDA(cudaGetLastError());
    const int wpb = 4;
    noise_compact_kernel<<<(unsigned)((w + wpb - 1) / wpb), 32 * wpb, 0, stream>>>(seg, w);
    PS_CUDA(cudaGetLastError());
    return OK;
}

int launch_segment(cudaStream_t stream, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, const SegmentDev &seg,
                   int rows, int bw, int threads, const u64 *const *recs) {
    const int64_t W = 2 * n + 1;
    const int64_t nchunks = (w + bw - 1) / bw;
    const int64_t tiles = ((W + rows - 1) / rows) * nchunks;
    const size_t smem =
        segment_launch_smem(seg.nlayers, seg.nruns, seg.ngates, seg.nsigns, seg.nq, seg.nrecsig, rows, bw);
    if (smem > kSegSmemMax) return fail(E_ARG, "segment tile does not fit in shared memory");
    if (threads % 32 != 0 || threads > 256 || bw > 32 || 32 % bw != 0)
        return fail(E_ARG, "segment tile: threads a multiple of 32 (at most 256), words a divisor of 32");
    {
        const int rc = allow_max_smem((const void *)segment_kernel);
        if (rc != OK) return rc;
    }
    if (g_num_sms == 0) {
        int dev = 0;
        PS_CUDA(cudaGetDevice(&dev));
        PS_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
    }
    int per_sm = 0;
    PS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, segment_kernel, threads, smem));
    if (per_sm < 1) return fail(E_ARG, "segment kernel does not fit on an SM");
    const int64_t grid = std::min<int64_t>(tiles, (int64_t)per_sm * g_num_sms);
    segment_kernel<<<(unsigned)grid, threads, smem, stream>>>(X, Z, R, n, W, w, seg, rows, bw, nchunks, tiles, recs);
    PS_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace ps
