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
            NoiseEntry e;
            e.fxa = fxa;
            e.fza = fza;
            e.fxb = fxb;
            e.fzb = fzb;
            e.slot = s;
            e.layer = seg.slots[s].layer;
            out[pos] = e;
        }
        count += __popc(bal);
    }
    if (lane == 0) seg.entry_count[k] = count;
}

__device__ __forceinline__ void apply_gate(const SegGate &g, u64 *__restrict__ xr, u64 *__restrict__ zr, u64 &rd,
                                           const u64 *const *__restrict__ recs, int64_t kg) {
    const int a = g.a;
    switch (g.code) {
    case OP_H: {  // GateFunctors.hpp:90-93
        const u64 x = xr[a], z = zr[a];
        rd ^= x & z;
        xr[a] = z;
        zr[a] = x;
        break;
    }
    case OP_S: {  // :165-169
        const u64 x = xr[a], z = zr[a];
        rd ^= x & z;
        zr[a] = z ^ x;
        break;
    }
    case OP_CX: {  // :248-253
        const int b = g.b;
        const u64 xc = xr[a], zc = zr[a], xt = xr[b], zt = zr[b];
        rd ^= xc & zt & ~(xt ^ zc);
        xr[b] = xt ^ xc;
        zr[a] = zc ^ zt;
        break;
    }
    case OP_CZ: {  // :30-35
        const int b = g.b;
        const u64 xc = xr[a], zc = zr[a], xt = xr[b], zt = zr[b];
        rd ^= xc & xt & (zt ^ zc);
        zr[b] = zt ^ xc;
        zr[a] = zc ^ xt;
        break;
    }
    case OP_H_IF: {  // :143-148
        const u64 f = recs[g.rec][kg];
        const u64 x = xr[a], z = zr[a];
        rd ^= f & x & z;
        xr[a] = (x & ~f) | (z & f);
        zr[a] = (z & ~f) | (x & f);
        break;
    }
    case OP_S_IF: {  // :221-228
        const u64 f = recs[g.rec][kg];
        const u64 x = xr[a], z = zr[a];
        rd ^= f & x & z;
        zr[a] = z ^ (f & x);
        break;
    }
    default: break;
    }
}

__global__ void __launch_bounds__(512) segment_kernel(u64 *__restrict__ X, u64 *__restrict__ Z, u64 *__restrict__ R,
                                                     int64_t n, int64_t W, int64_t w, SegmentDev seg, int rows,
                                                     int bw, int64_t nchunks, const u64 *const *__restrict__ recs) {
    extern __shared__ u64 sm[];
    const int nq = seg.nq;
    u64 *xs = sm;                             // [rows][bw][nq]
    u64 *zs = xs + (size_t)rows * bw * nq;    // [rows][bw][nq]
    u64 *rdel = zs + (size_t)rows * bw * nq;  // [rows][bw]
    const int64_t tile = blockIdx.x;
    const int64_t row0 = (tile / nchunks) * rows;
    const int64_t k0 = (tile % nchunks) * bw;
    const int T = blockDim.x, tid = threadIdx.x;
    const int half = bw >> 1;

    // ---- load (16-byte global loads, transposed into shared memory)
    const int items = rows * nq * half;
    for (int idx = tid; idx < items; idx += T) {
        const int k2 = idx % half;
        const int rest = idx / half;
        const int l = rest % nq, r = rest / nq;
        const int64_t row = row0 + r;
        const int64_t kg = k0 + 2 * k2;
        ulonglong2 vx = make_ulonglong2(0, 0), vz = make_ulonglong2(0, 0);
        if (row < W && kg < w) {
            const int64_t off = (row * n + seg.cols[l]) * w + kg;
            vx = *reinterpret_cast<const ulonglong2 *>(X + off);
            vz = *reinterpret_cast<const ulonglong2 *>(Z + off);
        }
        const int base = (r * bw + 2 * k2) * nq + l;
        xs[base] = vx.x;
        xs[base + nq] = vx.y;
        zs[base] = vz.x;
        zs[base + nq] = vz.y;
    }
    __syncthreads();

    // ---- apply the schedule: warp = (row, word)
    const int lane = tid & 31, wid = tid >> 5, nw = T >> 5;
    for (int pair = wid; pair < rows * bw; pair += nw) {
        const int r = pair / bw, kk = pair % bw;
        const int64_t row = row0 + r, kg = k0 + kk;
        u64 rd = 0ull;
        if (row < W && kg < w) {
            u64 *xr = xs + (size_t)pair * nq;
            u64 *zr = zs + (size_t)pair * nq;
            const NoiseEntry *ent = seg.entries ? seg.entries + kg * (int64_t)seg.cap : nullptr;
            const int nent = seg.entries ? seg.entry_count[kg] : 0;
            int cursor = 0;
            for (int L = 0; L < seg.nlayers; ++L) {
                const SegLayer ly = seg.layers[L];
                for (int g = ly.g0 + lane; g < ly.g1; g += 32) apply_gate(seg.gates[g], xr, zr, rd, recs, kg);
                __syncwarp();
                for (int s = ly.s0 + lane; s < ly.s1; s += 32) {
                    const SegSign sg = seg.signs[s];
                    const u64 x = xr[sg.a], z = zr[sg.a];
                    if (sg.kind == SIGN_X)
                        rd ^= z;
                    else if (sg.kind == SIGN_Y)
                        rd ^= x ^ z;
                    else if (sg.kind == SIGN_Z)
                        rd ^= x;
                    else
                        rd ^= recs[sg.rec][kg] & z;
                }
                // Channel outcomes of this layer (the list is in layer order).
                while (cursor < nent) {
                    const int e = cursor + lane;
                    const bool mine = e < nent && ent[e].layer == L;
                    const unsigned bal = __ballot_sync(0xffffffffu, mine);
                    if (mine) {
                        const NoiseEntry en = ent[e];
                        const NoiseSlot sl = seg.slots[en.slot];
                        rd ^= (en.fxa & zr[sl.a]) ^ (en.fza & xr[sl.a]);
                        if (sl.b >= 0) rd ^= (en.fxb & zr[sl.b]) ^ (en.fzb & xr[sl.b]);
                    }
                    const int c = __popc(bal);
                    cursor += c;
                    if (c < 32) break;
                }
                __syncwarp();
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) rd ^= __shfl_xor_sync(0xffffffffu, rd, off);
        if (lane == 0) rdel[pair] = rd;
    }
    __syncthreads();

    // ---- store back
    for (int idx = tid; idx < items; idx += T) {
        const int k2 = idx % half;
        const int rest = idx / half;
        const int l = rest % nq, r = rest / nq;
        const int64_t row = row0 + r;
        const int64_t kg = k0 + 2 * k2;
        if (row < W && kg < w) {
            const int base = (r * bw + 2 * k2) * nq + l;
            const int64_t off = (row * n + seg.cols[l]) * w + kg;
            *reinterpret_cast<ulonglong2 *>(X + off) = make_ulonglong2(xs[base], xs[base + nq]);
            *reinterpret_cast<ulonglong2 *>(Z + off) = make_ulonglong2(zs[base], zs[base + nq]);
        }
    }
    for (int pair = tid; pair < rows * bw; pair += T) {
        const int r = pair / bw, kk = pair % bw;
        const int64_t row = row0 + r, kg = k0 + kk;
        if (row < W && kg < w && rdel[pair]) R[row * w + kg] ^= rdel[pair];
    }
}

}  // namespace

size_t segment_smem_bytes(int nq, int rows, int bw) { return (size_t)rows * bw * (2 * (size_t)nq + 1) * sizeof(u64); }

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
    const size_t smem = segment_smem_bytes(seg.nq, rows, bw);
    if (smem > 227 * 1024) return fail(E_ARG, "segment tile does not fit in shared memory");
    if (smem > 48 * 1024)
        PS_CUDA(cudaFuncSetAttribute(segment_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    segment_kernel<<<(unsigned)tiles, threads, smem, stream>>>(X, Z, R, n, W, w, seg, rows, bw, nchunks, recs);
    PS_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace ps
