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

#include "ps_frame.h"
#include "ps_internal.h"
#include "ps_segment.cuh"

namespace ps {

namespace {

// Pauli-channel sampling for one segment, pass 1: one thread per (word,
// channel) draws the word's outcomes (channel_word) into dense[word][slot].
__global__ void __launch_bounds__(256) noise_dense_kernel(SegmentDev seg, int64_t w, const RunParams *__restrict__ rp) {
    const int64_t pair = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t k = pair / seg.nslots;
    const int s = (int)(pair - k * seg.nslots);
    if (k >= w) return;
    const NoiseSlot sl = seg.slots[s];
    const ChannelWord m = channel_word(rp->seed, rp->event_base + sl.event, rp->word_base + (uint64_t)k,
                                       seg.thr + sl.thr_off, sl.count);
    u64 *d = seg.dense + pair * 4;
    d[0] = m.fxa;
    d[1] = m.fza;
    d[2] = m.fxb;
    d[3] = m.fzb;
}

// Pass 2: one warp per word appends the non-identity outcomes to the word's
// entry list; ballot compaction keeps slot (= layer) order.
__global__ void __launch_bounds__(128) noise_compact_kernel(SegmentDev seg, int64_t w, int slot_tags) {
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
            e.layer = (seg.res_slots || slot_tags) ? s : sl.layer;  // resident form, shared x/z: the slot
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
// and every lane keeps GU independent gates in flight (gates g, g+32, ...),
// so their shared-memory loads overlap.
template <int CODE>
__device__ __forceinline__ void layer_uniform(const SegGate *__restrict__ gates, int g0, int g1, int lane,
                                              XZ *__restrict__ t, u64 &rd) {
    constexpr int GU = 4;
    for (int g = g0 + lane; g < g1; g += 32 * GU) {
        SegGate gg[GU];
        bool on[GU];
#pragma unroll
        for (int u = 0; u < GU; ++u) {
            on[u] = g + 32 * u < g1;
            gg[u] = gates[on[u] ? g + 32 * u : g];
        }
        if (CODE == OP_H || CODE == OP_S) {
            XZ v[GU];
#pragma unroll
            for (int u = 0; u < GU; ++u) v[u] = t[gg[u].a];
#pragma unroll
            for (int u = 0; u < GU; ++u)
                if (on[u]) {
                    rd ^= v[u].x & v[u].y;
                    t[gg[u].a] = CODE == OP_H ? make_ulonglong2(v[u].y, v[u].x)
                                              : make_ulonglong2(v[u].x, v[u].y ^ v[u].x);
                }
        } else {
            XZ c[GU], u2[GU];
#pragma unroll
            for (int u = 0; u < GU; ++u) {
                c[u] = t[gg[u].a];
                u2[u] = t[gg[u].b];
            }
#pragma unroll
            for (int u = 0; u < GU; ++u)
                if (on[u]) {
                    if (CODE == OP_CX) {
                        rd ^= c[u].x & u2[u].y & ~(u2[u].x ^ c[u].y);
                        t[gg[u].b] = make_ulonglong2(u2[u].x ^ c[u].x, u2[u].y);
                        t[gg[u].a] = make_ulonglong2(c[u].x, c[u].y ^ u2[u].y);
                    } else {
                        rd ^= c[u].x & u2[u].x & (u2[u].y ^ c[u].y);
                        t[gg[u].b] = make_ulonglong2(u2[u].x, u2[u].y ^ c[u].x);
                        t[gg[u].a] = make_ulonglong2(c[u].x, c[u].y ^ u2[u].x);
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

// Parity of [row anticommutes with propagated Pauli pid] per shot bit, from
// the row's final cells.
__device__ __forceinline__ u64 prop_parity(const SegmentDev &seg, int pid, const XZ *__restrict__ t) {
    const uint32_t desc = __ldg(seg.prop_desc + pid);
    const uint32_t off = desc >> 8, len = desc & 255u;
    u64 par = 0ull;
    for (uint32_t k = 0; k < len; ++k) {
        const uint32_t u = __ldg(seg.prop_sup + off + k);
        const XZ v = t[u & 0xFFFFu];
        if (u & PROP_Z) par ^= v.x;
        if (u & PROP_X) par ^= v.y;
    }
    return par;
}

// Resident steps of one layer for RC register slots, CH slots at a time:
// all partner cells of a chunk are loaded before any is written (the gates of
// one layer act on distinct columns), so the loads overlap.
template <int RC>
__device__ __forceinline__ void resident_layer(const ResOp *__restrict__ ops, int lane, XZ *__restrict__ t,
                                               u64 (&xr)[RC], u64 (&zr)[RC], u64 &rd) {
    constexpr int CH = RC < 4 ? RC : 4;
#pragma unroll
    for (int j0 = 0; j0 < RC; j0 += CH) {
        ResOp op[CH];
        XZ v[CH];
#pragma unroll
        for (int u = 0; u < CH; ++u) {
            op[u] = ops[(j0 + u) * 32 + lane];
            v[u] = op[u].code >= RS_CX_CTRL ? t[op[u].other] : make_ulonglong2(0ull, 0ull);
        }
#pragma unroll
        for (int u = 0; u < CH; ++u) {
            const int j = j0 + u;
            u64 &x = xr[j], &z = zr[j];
            switch (op[u].code) {
            case RS_H: {  // GateFunctors.hpp:90-93
                rd ^= x & z;
                const u64 tmp = x;
                x = z;
                z = tmp;
                break;
            }
            case RS_S:  // :165-169
                rd ^= x & z;
                z ^= x;
                break;
            case RS_CX_CTRL:  // :248-253, resident = control
                rd ^= x & v[u].y & ~(v[u].x ^ z);
                t[op[u].other] = make_ulonglong2(v[u].x ^ x, v[u].y);
                z ^= v[u].y;
                break;
            case RS_CX_TGT:  // resident = target
                rd ^= v[u].x & z & ~(x ^ v[u].y);
                t[op[u].other] = make_ulonglong2(v[u].x, v[u].y ^ z);
                x ^= v[u].x;
                break;
            case RS_CZ:  // :30-35
                rd ^= x & v[u].x & (v[u].y ^ z);
                t[op[u].other] = make_ulonglong2(v[u].x, v[u].y ^ x);
                z ^= v[u].x;
                break;
            default: break;
            }
        }
    }
}

// Word-vector form: thread = gate, looping over the tile's PB words (tile
// rows p = 0..PB-1): the gate is decoded once for all words, and the cell
// loads of CH words are in flight together.  The schedule is read through L1
// (every CTA reads the same gates), leaving shared memory to the tile.
template <int CODE, int PB>
__device__ __forceinline__ void gates_wv(const SegGate *__restrict__ gates, int g0, int g1, int tid, int T,
                                         XZ *__restrict__ tile, int nq1, u64 (&rd)[PB]) {
    constexpr int CH = PB < 4 ? PB : 4;
    for (int g = g0 + tid; g < g1; g += T) {
        const SegGate gg = gates[g];
#pragma unroll
        for (int p0 = 0; p0 < PB; p0 += CH) {
            if (CODE == OP_H || CODE == OP_S) {
                XZ v[CH];
#pragma unroll
                for (int q = 0; q < CH; ++q) v[q] = tile[(p0 + q) * nq1 + gg.a];
#pragma unroll
                for (int q = 0; q < CH; ++q) {
                    rd[p0 + q] ^= v[q].x & v[q].y;
                    tile[(p0 + q) * nq1 + gg.a] = CODE == OP_H ? make_ulonglong2(v[q].y, v[q].x)
                                                               : make_ulonglong2(v[q].x, v[q].y ^ v[q].x);
                }
            } else {
                XZ c[CH], u[CH];
#pragma unroll
                for (int q = 0; q < CH; ++q) {
                    c[q] = tile[(p0 + q) * nq1 + gg.a];
                    u[q] = tile[(p0 + q) * nq1 + gg.b];
                }
#pragma unroll
                for (int q = 0; q < CH; ++q) {
                    const int p = p0 + q;
                    if (CODE == OP_CX) {  // GateFunctors.hpp:248-253
                        rd[p] ^= c[q].x & u[q].y & ~(u[q].x ^ c[q].y);
                        tile[p * nq1 + gg.b] = make_ulonglong2(u[q].x ^ c[q].x, u[q].y);
                        tile[p * nq1 + gg.a] = make_ulonglong2(c[q].x, c[q].y ^ u[q].y);
                    } else {  // CZ, :30-35
                        rd[p] ^= c[q].x & u[q].x & (u[q].y ^ c[q].y);
                        tile[p * nq1 + gg.b] = make_ulonglong2(u[q].x, u[q].y ^ c[q].x);
                        tile[p * nq1 + gg.a] = make_ulonglong2(c[q].x, c[q].y ^ u[q].x);
                    }
                }
            }
        }
    }
}

// Persistent: each CTA stages the segment's schedule and column map in shared
// memory once, then loops over tiles (ROWS rows x BW words x nq columns):
// stage the tile, apply the schedule (one warp per (row, word)), store back.
// RC = 0: every gate reads and writes its cells in shared memory, channel
// outcomes and sign ops act at their layer.  RC > 0: the resident form.
// PB > 0 (RC = 0, one tile row of PB words): the word-vector form, threads
// spread over the gates of a layer instead of warps over (row, word) pairs.
template <int RC, int PB = 0>
__global__ void __launch_bounds__(256, 2) segment_kernel(u64 *__restrict__ X, u64 *__restrict__ Z,
                                                        u64 *__restrict__ R, int64_t n, int64_t W, int64_t w,
                                                        SegmentDev seg, int rows, int bw, int64_t nchunks,
                                                        int64_t ntiles, const u64 *const *__restrict__ recs) {
    extern __shared__ u64 sm[];
    const int nq = seg.nq;
    const int T = blockDim.x, tid = threadIdx.x;
    const int nq1 = seg_row_cells(nq);
    SegLayer *s_layers = reinterpret_cast<SegLayer *>(sm);
    SegRun *s_runs = reinterpret_cast<SegRun *>(s_layers + seg.nlayers);
    SegGate *s_gates = reinterpret_cast<SegGate *>(s_runs + seg.nruns);
    const int ngates_sm = PB > 0 ? 0 : seg.ngates;  // the word-vector form reads gates through L1
    SegSign *s_signs = reinterpret_cast<SegSign *>(s_gates + ngates_sm);
    int32_t *s_cols = reinterpret_cast<int32_t *>(s_signs + seg.nsigns);
    const int nres_ops = RC ? seg.nlayers * RC * 32 : 0;
    ResOp *s_resops = reinterpret_cast<ResOp *>(s_cols + nq);                   // [nlayers][RC][32]
    uint16_t *s_rescols = reinterpret_cast<uint16_t *>(s_resops + nres_ops);    // [RC][32]
    const size_t head = ((size_t)seg.nlayers * sizeof(SegLayer) + (size_t)seg.nruns * sizeof(SegRun) +
                         (size_t)ngates_sm * sizeof(SegGate) + (size_t)seg.nsigns * sizeof(SegSign) +
                         (size_t)nq * sizeof(int32_t) + (size_t)nres_ops * sizeof(ResOp) +
                         (size_t)RC * 32 * sizeof(uint16_t) + 15) / 16 * 2;
    const u64 **s_recp = reinterpret_cast<const u64 **>(sm + head);  // [nrecsig] record pointers
    XZ *tile_xz = reinterpret_cast<XZ *>(sm + head + (seg.nrecsig + 1) / 2 * 2);  // [rows*bw][nq1]
    u64 *rtile = reinterpret_cast<u64 *>(tile_xz + (size_t)rows * bw * nq1);      // [rows*bw] r words
    u64 *s_recw = rtile + rows * bw;                                               // [bw][rs]
    const int rs = seg_rec_stride(seg.nrecsig, bw);
    for (int i = tid; i < seg.nrecsig; i += T) s_recp[i] = recs[seg.recsig_rec[i]];
    for (int i = tid; i < seg.nlayers; i += T) s_layers[i] = seg.layers[i];
    for (int i = tid; i < seg.nruns; i += T) s_runs[i] = seg.runs[i];
    for (int i = tid; i < ngates_sm; i += T) s_gates[i] = seg.gates[i];
    for (int i = tid; i < seg.nsigns; i += T) s_signs[i] = seg.signs[i];
    for (int i = tid; i < nq; i += T) s_cols[i] = seg.cols[i];
    for (int i = tid; i < nres_ops; i += T) s_resops[i] = seg.res_ops[i];
    for (int i = tid; i < RC * 32; i += T) s_rescols[i] = seg.res_cols[i];
    __syncthreads();

    const int lane = tid & 31, wid = tid >> 5, nw = T >> 5;
    // Staging map: lane -> word pair kp (words 2kp, 2kp+1) and column slot
    // jl.  A lane reads the 16-byte x and z chunks of its two words (two
    // global loads) and writes two whole {x, z} cells (two 16-byte shared
    // stores).  A quarter-warp's 8 cells fall on distinct bank groups (the
    // tile row stride nq1 is odd and the word offsets 2kp are even), so each
    // store is one wavefront per quarter-warp; the loads stay coalesced.
    const int npair = bw >= 2 ? bw / 2 : 1;          // word pairs per tile row
    const int kp = lane % npair, jl = lane / npair;  // jl < 32 / npair
    const int jln = 32 / npair;                      // columns per instruction
    constexpr int SU = 4;                            // columns in flight per lane
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t row0 = (tile / nchunks) * rows;
        const int64_t k0 = (tile % nchunks) * bw;
        // ---- load
        for (int e = tid; e < rows * bw * kSegDummyCols; e += T)
            tile_xz[(size_t)(e / kSegDummyCols) * nq1 + nq + e % kSegDummyCols] = make_ulonglong2(0ull, 0ull);
        for (int r = 0; r < rows; ++r) {
            const int64_t row = row0 + r;
            const int64_t kg = k0 + 2 * kp;  // first word of the lane's pair
            const bool ok0 = row < W && kg < w, ok1 = bw >= 2 && row < W && kg + 1 < w;
            XZ *d0 = tile_xz + (size_t)(r * bw + 2 * kp) * nq1;
            XZ *d1 = d0 + nq1;
            const int64_t rbase = row * n * w + kg;
            for (int cb = wid * jln * SU; cb < nq; cb += nw * jln * SU) {
                ulonglong2 xv[SU], zv[SU];
#pragma unroll
                for (int u = 0; u < SU; ++u) {
                    const int l = cb + u * jln + jl;
                    xv[u] = zv[u] = make_ulonglong2(0ull, 0ull);
                    if (l < nq && ok0) {
                        const int64_t off = rbase + (int64_t)s_cols[l] * w;
                        if (ok1) {  // kg even and w even: 16-byte aligned
                            xv[u] = *reinterpret_cast<const ulonglong2 *>(X + off);
                            zv[u] = *reinterpret_cast<const ulonglong2 *>(Z + off);
                        } else {
                            xv[u].x = X[off];
                            zv[u].x = Z[off];
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < SU; ++u) {
                    const int l = cb + u * jln + jl;
                    if (l < nq && 2 * kp < bw) {
                        d0[l] = make_ulonglong2(xv[u].x, zv[u].x);
                        if (bw >= 2) d1[l] = make_ulonglong2(xv[u].y, zv[u].y);
                    }
                }
            }
        }
        for (int pair = tid; pair < rows * bw; pair += T) {
            const int64_t row = row0 + pair / bw, kg = k0 + pair % bw;
            if (row < W && kg < w) cp_async8(&rtile[pair], R + row * w + kg);
        }
        {  // bw is a power of two dividing T: a thread copies one word of records
            const int kk = tid & (bw - 1);
            const int64_t kg = k0 + kk;
            if (kg < w)
                for (int slot = tid / bw; slot < seg.nrecsig; slot += T / bw)
                    cp_async8(&s_recw[kk * rs + slot], s_recp[slot] + kg);
        }
        cp_async_wait_all();
        __syncthreads();

        if constexpr (PB > 0) {
            // ---- apply the schedule: thread = gate, all PB words of the tile
            __shared__ u64 s_rdx[PB > 0 ? PB : 1];
            __shared__ int s_eoff[PB + 1];
            if (tid < PB) s_rdx[tid] = 0ull;
            if (tid == 0) {
                int acc = 0;
#pragma unroll
                for (int p = 0; p < PB; ++p) {
                    s_eoff[p] = acc;
                    const int64_t kg = k0 + p;
                    acc += (seg.entries && kg < w) ? seg.entry_count[kg] : 0;
                }
                s_eoff[PB] = acc;
            }
            __syncthreads();
            const int ntot = s_eoff[PB];
            u64 rd[PB > 0 ? PB : 1];
#pragma unroll
            for (int p = 0; p < PB; ++p) rd[p] = 0ull;
            // channel outcomes of the tile's words: item i -> (word p, entry)
            constexpr int NEI = 3;
            NoiseEntry mine[NEI];
            int mp[NEI];
#pragma unroll
            for (int u = 0; u < NEI; ++u) {
                const int it = tid + u * T;
                mine[u].layer = -1;
                mp[u] = 0;
                if (it < ntot) {
                    int p = 0;
                    while (p + 1 < PB && s_eoff[p + 1] <= it) ++p;
                    mine[u] = seg.entries[(k0 + p) * (int64_t)seg.cap + (it - s_eoff[p])];
                    mp[u] = p;
                }
            }
            const bool spill = ntot > NEI * T;
            const SegGate *__restrict__ gsched = seg.gates;
            for (int L = 0; L < seg.nlayers; ++L) {
                const SegLayer ly = s_layers[L];
                for (int ri = ly.r0; ri < ly.r1; ++ri) {  // runs touch disjoint columns
                    const SegRun rn = s_runs[ri];
                    switch (rn.code) {
                    case OP_H: gates_wv<OP_H, PB>(gsched, rn.g0, rn.g1, tid, T, tile_xz, nq1, rd); break;
                    case OP_S: gates_wv<OP_S, PB>(gsched, rn.g0, rn.g1, tid, T, tile_xz, nq1, rd); break;
                    case OP_CX: gates_wv<OP_CX, PB>(gsched, rn.g0, rn.g1, tid, T, tile_xz, nq1, rd); break;
                    case OP_CZ: gates_wv<OP_CZ, PB>(gsched, rn.g0, rn.g1, tid, T, tile_xz, nq1, rd); break;
                    default:
                        for (int g = rn.g0 + tid; g < rn.g1; g += T) {
                            const SegGate gg = gsched[g];
#pragma unroll
                            for (int p = 0; p < PB; ++p)
                                if (k0 + p < w) apply_gate(gg, tile_xz + p * nq1, rd[p], recs, k0 + p);
                        }
                    }
                }
                __syncthreads();
                // sign ops and channel outcomes after this layer's gates (reads only)
                for (int si = ly.s0 + tid; si < ly.s1; si += T) {
                    const SegSign sg = s_signs[si];
#pragma unroll
                    for (int p = 0; p < PB; ++p) {
                        const XZ v = tile_xz[p * nq1 + sg.a];
                        if (sg.kind == SIGN_X)
                            rd[p] ^= v.y;
                        else if (sg.kind == SIGN_Y)
                            rd[p] ^= v.x ^ v.y;
                        else if (sg.kind == SIGN_Z)
                            rd[p] ^= v.x;
                        else
                            rd[p] ^= s_recw[p * rs + sg.rec] & v.y;
                    }
                }
#pragma unroll
                for (int u = 0; u < NEI; ++u)
                    if (mine[u].layer == L) {
                        u64 c = 0ull;
                        apply_entry(mine[u], tile_xz + mp[u] * nq1, c);
                        if (c) atomicXor(&s_rdx[mp[u]], c);
                    }
                if (spill) {  // more outcomes than the registers hold
                    for (int it = NEI * T + tid; it < ntot; it += T) {
                        int p = 0;
                        while (p + 1 < PB && s_eoff[p + 1] <= it) ++p;
                        const NoiseEntry en = seg.entries[(k0 + p) * (int64_t)seg.cap + (it - s_eoff[p])];
                        if (en.layer != L) continue;
                        u64 c = 0ull;
                        apply_entry(en, tile_xz + p * nq1, c);
                        if (c) atomicXor(&s_rdx[p], c);
                    }
                }
                __syncthreads();
            }
            // r: every thread's accumulators, reduced per word
#pragma unroll
            for (int p = 0; p < PB; ++p) {
                u64 v = rd[p];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) v ^= __shfl_xor_sync(0xffffffffu, v, off);
                if (lane == 0 && v) atomicXor(&s_rdx[p], v);
            }
            __syncthreads();
            if (tid < PB) rtile[tid] ^= s_rdx[tid];
            __syncthreads();
        } else {
        // ---- apply the schedule: warp = (row, word)
        for (int pair = wid; pair < rows * bw; pair += nw) {
            const int r = pair / bw, kk = pair % bw;
            const int64_t row = row0 + r, kg = k0 + kk;
            u64 rd = 0ull;
            if (RC == 0 && row < W && kg < w) {
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
                            rd ^= s_recw[kk * rs + sg.rec] & v.y;
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
            if (RC > 0 && row < W && kg < w) {
                XZ *t = tile_xz + (size_t)pair * nq1;
                u64 xr[RC > 0 ? RC : 1], zr[RC > 0 ? RC : 1];
#pragma unroll
                for (int j = 0; j < RC; ++j) {
                    const uint16_t c = s_rescols[j * 32 + lane];
                    const XZ v = c != 0xFFFFu ? t[c] : make_ulonglong2(0ull, 0ull);
                    xr[j] = v.x;
                    zr[j] = v.y;
                }
                for (int L = 0; L < seg.nlayers; ++L) {
                    if constexpr (RC > 0) resident_layer<RC>(s_resops + L * RC * 32, lane, t, xr, zr, rd);
                    const SegLayer ly = s_layers[L];
                    for (int ri = ly.r0; ri < ly.r1; ++ri) {  // gates without resident columns
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
                }
#pragma unroll
                for (int j = 0; j < RC; ++j) {
                    const uint16_t c = s_rescols[j * 32 + lane];
                    if (c != 0xFFFFu) t[c] = make_ulonglong2(xr[j], zr[j]);
                }
                __syncwarp();
                // Sign ops and channel outcomes after the last layer, through
                // their propagated Paulis.
                const int nsg = seg.nsigns;
                const NoiseEntry *ent = seg.entries ? seg.entries + kg * (int64_t)seg.cap : nullptr;
                const int nent = seg.entries ? seg.entry_count[kg] : 0;
                const int pbase = 4 * seg.nslots;
                for (int it = lane; it < nsg + nent; it += 32) {
                    if (it < nsg) {
                        const SegSign sg = s_signs[it];
                        const u64 m = sg.kind == SIGN_REC_X ? s_recw[kk * rs + sg.rec] : ~0ull;
                        if (m) rd ^= m & prop_parity(seg, pbase + it, t);
                    } else {
                        const NoiseEntry e = ent[it - nsg];
                        const int sb = 4 * e.layer;  // resident form: the channel's slot
                        if (e.fxa) rd ^= e.fxa & prop_parity(seg, sb + 0, t);
                        if (e.fza) rd ^= e.fza & prop_parity(seg, sb + 1, t);
                        if (e.fxb) rd ^= e.fxb & prop_parity(seg, sb + 2, t);
                        if (e.fzb) rd ^= e.fzb & prop_parity(seg, sb + 3, t);
                    }
                }
                __syncwarp();
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) rd ^= __shfl_xor_sync(0xffffffffu, rd, off);
            if (lane == 0) rtile[pair] ^= rd;
        }
        __syncthreads();

        }
        // ---- store back (the staging map in reverse: two cells -> 16-byte x
        // and z chunks of a word pair)
        for (int r = 0; r < rows; ++r) {
            const int64_t row = row0 + r;
            const int64_t kg = k0 + 2 * kp;
            if (!(row < W && kg < w)) continue;
            const bool two = bw >= 2;
            const XZ *d0 = tile_xz + (size_t)(r * bw + 2 * kp) * nq1;
            const XZ *d1 = d0 + nq1;
            const int64_t rbase = row * n * w + kg;
            for (int cb = wid * jln; cb < nq; cb += nw * jln) {
                const int l = cb + jl;
                if (l >= nq) continue;
                const int64_t off = rbase + (int64_t)s_cols[l] * w;
                const XZ a = d0[l];
                if (two) {
                    const XZ b = d1[l];
                    *reinterpret_cast<ulonglong2 *>(X + off) = make_ulonglong2(a.x, b.x);
                    *reinterpret_cast<ulonglong2 *>(Z + off) = make_ulonglong2(a.y, b.y);
                } else {
                    X[off] = a.x;
                    Z[off] = a.y;
                }
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

size_t segment_smem_bytes(int nq, int rows, int bw) {
    return (size_t)rows * bw * (2 * (size_t)seg_row_cells(nq) + 1) * sizeof(u64);
}

size_t segment_launch_smem(int nlayers, int nruns, int ngates, int nsigns, int nq, int nrecsig, int rows, int bw,
                           int rc) {
    const size_t sched = ((size_t)nlayers * sizeof(SegLayer) + (size_t)nruns * sizeof(SegRun) +
                          (size_t)ngates * sizeof(SegGate) + (size_t)nsigns * sizeof(SegSign) +
                          (size_t)nq * sizeof(int32_t) + (size_t)nlayers * rc * 32 * sizeof(ResOp) +
                          (size_t)rc * 32 * sizeof(uint16_t) + 15) / 16 * 16 +
                         (size_t)(nrecsig + 1) / 2 * 16 + (size_t)seg_rec_stride(nrecsig, bw) * bw * 8 +
                         (size_t)rows * bw * 8;
    return segment_smem_bytes(nq, rows, bw) + sched;
}

int launch_noise_sample(cudaStream_t stream, const SegmentDev &seg, int64_t w, const RunParams *rp, int slot_tags) {
    if (seg.nslots == 0) return OK;
    const int64_t threads = (int64_t)seg.nslots * w;
    noise_dense_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, stream>>>(seg, w, rp);
    PS_CUDA(cudaGetLastError());
    const int wpb = 4;
    noise_compact_kernel<<<(unsigned)((w + wpb - 1) / wpb), 32 * wpb, 0, stream>>>(seg, w, slot_tags);
    PS_CUDA(cudaGetLastError());
    return OK;
}

namespace {
template <int RC, int PB>
int launch_segment_rc(cudaStream_t stream, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, const SegmentDev &seg,
                      int rows, int bw, int threads, const u64 *const *recs, size_t smem) {
    const int64_t W = 2 * n + 1;
    const int64_t nchunks = (w + bw - 1) / bw;
    const int64_t tiles = ((W + rows - 1) / rows) * nchunks;
    {
        const int rc = allow_max_smem((const void *)segment_kernel<RC, PB>);
        if (rc != OK) return rc;
    }
    if (g_num_sms == 0) {
        int dev = 0;
        PS_CUDA(cudaGetDevice(&dev));
        PS_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
    }
    int per_sm = 0;
    PS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, segment_kernel<RC, PB>, threads, smem));
    if (per_sm < 1) return fail(E_ARG, "segment kernel does not fit on an SM");
    const int64_t grid = std::min<int64_t>(tiles, (int64_t)per_sm * g_num_sms);
    segment_kernel<RC, PB><<<(unsigned)grid, threads, smem, stream>>>(X, Z, R, n, W, w, seg, rows, bw, nchunks, tiles,
                                                                   recs);
    PS_CUDA(cudaGetLastError());
    return OK;
}
}  // namespace

int launch_segment(cudaStream_t stream, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t w, const SegmentDev &seg,
                   int rows, int bw, int threads, const u64 *const *recs) {
    const bool wv = seg.word_vector && rows == 1 && seg.res_slots == 0;
    const size_t smem = segment_launch_smem(seg.nlayers, seg.nruns, wv ? 0 : seg.ngates, seg.nsigns, seg.nq,
                                            seg.nrecsig, rows, bw, seg.res_slots);
    if (smem > kSegSmemMax) return fail(E_ARG, "segment tile does not fit in shared memory");
    if (threads % 32 != 0 || threads > 256 || bw > 16 || 16 % bw != 0)
        return fail(E_ARG, "segment tile: threads a multiple of 32 (at most 256), words a divisor of 16");
    switch (seg.res_slots) {
    case 0:
        if (seg.word_vector && rows == 1) switch (bw) {  // the word-vector form
            case 1: return launch_segment_rc<0, 1>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
            case 2: return launch_segment_rc<0, 2>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
            case 4: return launch_segment_rc<0, 4>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
            case 8: return launch_segment_rc<0, 8>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
            case 16: return launch_segment_rc<0, 16>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
            default: break;
            }
        return launch_segment_rc<0, 0>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
    case 2: return launch_segment_rc<2, 0>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
    case 4: return launch_segment_rc<4, 0>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
    case 8: return launch_segment_rc<8, 0>(stream, X, Z, R, n, w, seg, rows, bw, threads, recs, smem);
    default: return fail(E_ARG, "resident slots per lane must be 0, 2, 4 or 8");
    }
}

}  // namespace ps
