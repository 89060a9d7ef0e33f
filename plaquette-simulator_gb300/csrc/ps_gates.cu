// ps_gates.cu -- the plain per-gate form: one launch per gate (or per Pauli
// channel), each a coalesced 128-bit pass over the touched tableau columns
// of all W rows.  This is the drop-in for the reference's per-gate
// parallel_for launches (CliffordState.hpp:348-531) and the baseline the
// fused circuit form is measured against.
#include <cuda.h>

#include <cmath>
#include <mutex>
#include <string>

#include "ps_internal.h"
#include "ps_segment.cuh"

namespace ps {

namespace {

struct W2 {
    u64 a, b;
};

__device__ __forceinline__ W2 ld2(const u64 *p) {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(p);
    return {v.x, v.y};
}
__device__ __forceinline__ void st2(u64 *p, u64 a, u64 b) {
    *reinterpret_cast<ulonglong2 *>(p) = make_ulonglong2(a, b);
}

// Per-word gate algebra (GateFunctors.hpp), 64 shots at a time.
template <int CODE>
__device__ __forceinline__ void apply_1q(u64 &x, u64 &z, u64 &r, u64 f) {
    if (CODE == OP_H) {  // GateFunctors.hpp:90-93
        r ^= x & z;
        const u64 t = x;
        x = z;
        z = t;
    } else if (CODE == OP_S) {  // :165-169
        r ^= x & z;
        z ^= x;
    } else if (CODE == OP_X) {  // :304-307
        r ^= z;
    } else if (CODE == OP_Y) {  // :324-327
        r ^= x ^ z;
    } else if (CODE == OP_Z) {  // :373-376
        r ^= x;
    } else if (CODE == OP_H_IF) {  // :143-148, per-shot flag f
        r ^= f & x & z;
        const u64 nx = (x & ~f) | (z & f);
        z = (z & ~f) | (x & f);
        x = nx;
    } else if (CODE == OP_S_IF) {  // :221-228
        r ^= f & x & z;
        z ^= f & x;
    }
}

// One thread per (row, pair of shot-words): W * w/2 threads.
template <int CODE>
__global__ void __launch_bounds__(256) gate1_kernel(u64 *__restrict__ X, u64 *__restrict__ Z, u64 *__restrict__ R,
                                                   int64_t n, int64_t W, int64_t w, int64_t q,
                                                   const u64 *__restrict__ flag) {
    const int64_t half = w >> 1;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * half) return;
    const int64_t i = idx / half, k = (idx - i * half) * 2;
    const int64_t off = (i * n + q) * w + k;
    W2 x = ld2(X + off), z = ld2(Z + off), r = ld2(R + i * w + k);
    u64 f0 = 0, f1 = 0;
    if (CODE == OP_H_IF || CODE == OP_S_IF) {
        const W2 f = ld2(flag + k);
        f0 = f.a;
        f1 = f.b;
    }
    apply_1q<CODE>(x.a, z.a, r.a, f0);
    apply_1q<CODE>(x.b, z.b, r.b, f1);
    if (CODE == OP_H || CODE == OP_H_IF || CODE == OP_S || CODE == OP_S_IF) {
        st2(X + off, x.a, x.b);
        st2(Z + off, z.a, z.b);
    }
    st2(R + i * w + k, r.a, r.b);
}

// CX (GateFunctors.hpp:248-253) and CZ (:30-35).
template <int CODE>
__global__ void __launch_bounds__(256) gate2_kernel(u64 *__restrict__ X, u64 *__restrict__ Z, u64 *__restrict__ R,
                                                   int64_t n, int64_t W, int64_t w, int64_t c, int64_t t) {
    const int64_t half = w >> 1;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * half) return;
    const int64_t i = idx / half, k = (idx - i * half) * 2;
    const int64_t oc = (i * n + c) * w + k, ot = (i * n + t) * w + k;
    W2 xc = ld2(X + oc), zc = ld2(Z + oc), xt = ld2(X + ot), zt = ld2(Z + ot), r = ld2(R + i * w + k);
    if (CODE == OP_CX) {
        r.a ^= xc.a & zt.a & ~(xt.a ^ zc.a);
        r.b ^= xc.b & zt.b & ~(xt.b ^ zc.b);
        st2(X + ot, xt.a ^ xc.a, xt.b ^ xc.b);
        st2(Z + oc, zc.a ^ zt.a, zc.b ^ zt.b);
    } else {
        r.a ^= xc.a & xt.a & (zt.a ^ zc.a);
        r.b ^= xc.b & xt.b & (zt.b ^ zc.b);
        st2(Z + ot, zt.a ^ xc.a, zt.b ^ xc.b);
        st2(Z + oc, zc.a ^ xt.a, zc.b ^ xt.b);
    }
    st2(R + i * w + k, r.a, r.b);
}

// Pauli-channel sampling: one thread per shot-word draws the word's
// outcomes (channel_word) and writes its masks: fx = shots with X or Y,
// fz = Y or Z, for qubit a (masks[0..w), [w..2w)) and b ([2w..3w), [3w..4w)).
__global__ void __launch_bounds__(256) channel_sample_kernel(u64 *__restrict__ masks, int64_t w, uint64_t seed_arg,
                                                            uint64_t event_arg, uint64_t word_base_arg,
                                                            const RunParams *__restrict__ rp,
                                                            int count, const uint64_t *__restrict__ thr) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= w) return;
    const uint64_t seed = rp ? rp->seed : seed_arg;
    const uint64_t event = (rp ? rp->event_base : 0ull) + event_arg;
    const uint64_t word_base = rp ? rp->word_base : word_base_arg;
    const ChannelWord m = channel_word(seed, event, word_base + (uint64_t)k, thr, count);
    masks[k] = m.fxa;
    masks[w + k] = m.fza;
    masks[2 * w + k] = m.fxb;
    masks[3 * w + k] = m.fzb;
}

// r ^= (fx & z_q) ^ (fz & x_q) over all rows: X flips rows with Z on q, Z
// flips rows with X on q (the reference's Pauli functors, GateFunctors.hpp:
// 303-307 and :372-376, applied per shot).
__global__ void __launch_bounds__(256) sign_flip_kernel(const u64 *__restrict__ X, const u64 *__restrict__ Z,
                                                       u64 *__restrict__ R, int64_t n, int64_t W, int64_t w,
                                                       int64_t q, const u64 *__restrict__ fx,
                                                       const u64 *__restrict__ fz) {
    const int64_t half = w >> 1;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W * half) return;
    const int64_t i = idx / half, k = (idx - i * half) * 2;
    const int64_t off = (i * n + q) * w + k;
    const W2 x = ld2(X + off), z = ld2(Z + off), a = ld2(fx + k), b = ld2(fz + k);
    W2 r = ld2(R + i * w + k);
    r.a ^= (a.a & z.a) ^ (b.a & x.a);
    r.b ^= (a.b & z.b) ^ (b.b & x.b);
    st2(R + i * w + k, r.a, r.b);
}

// The per-op channel of compiled plain runs in one launch: a CTA takes 8
// shot-words and a block of 64 rows, samples the words first
// (channel_word_est: the same draws as every other form; threads 0..7; the
// CTAs of other row blocks draw the same), then flips their signs over its
// rows, two words a thread (16-byte accesses, four threads a row).
template <int TWO>
__global__ void __launch_bounds__(256) channel_apply_kernel(const u64 *__restrict__ X, const u64 *__restrict__ Z,
                                                           u64 *__restrict__ R, int64_t n, int64_t W, int64_t w,
                                                           int64_t a, int64_t b, uint32_t event_off,
                                                           const RunParams *__restrict__ rp,
                                                           const uint64_t *__restrict__ thr, int count,
                                                           const uint32_t *__restrict__ surv, ChannelEst est) {
    __shared__ u64 sm[4][8];
    const int64_t k0 = (int64_t)blockIdx.x * 8;
    const int t = threadIdx.x;
    if (t < 8) {
        ChannelWord m{0ull, 0ull, 0ull, 0ull};
        if (k0 + t < w)
            m = channel_word_est(rp->seed, rp->event_base + event_off, rp->word_base + (uint64_t)(k0 + t), thr, count,
                                 surv, est);
        sm[0][t] = m.fxa;
        sm[1][t] = m.fza;
        sm[2][t] = m.fxb;
        sm[3][t] = m.fzb;
    }
    __syncthreads();
    const int64_t i0 = (int64_t)blockIdx.y * 64, i1 = i0 + 64 < W ? i0 + 64 : W;
    for (int64_t it = t; it < (i1 - i0) * 4; it += blockDim.x) {
        const int64_t i = i0 + (it >> 2);
        const int p = (int)(it & 3);
        const int64_t k = k0 + 2 * p;
        if (k >= w) continue;
        W2 r = ld2(R + i * w + k);
        const int64_t oa = (i * n + a) * w + k;
        const W2 xa = ld2(X + oa), za = ld2(Z + oa);
        r.a ^= (sm[0][2 * p] & za.a) ^ (sm[1][2 * p] & xa.a);
        r.b ^= (sm[0][2 * p + 1] & za.b) ^ (sm[1][2 * p + 1] & xa.b);
        if (TWO) {
            const int64_t ob = (i * n + b) * w + k;
            const W2 xb = ld2(X + ob), zb = ld2(Z + ob);
            r.a ^= (sm[2][2 * p] & zb.a) ^ (sm[3][2 * p] & xb.a);
            r.b ^= (sm[2][2 * p + 1] & zb.b) ^ (sm[3][2 * p + 1] & xb.b);
        }
        st2(R + i * w + k, r.a, r.b);
    }
}

inline int blocks_for(int64_t threads) { return (int)((threads + 255) / 256); }

}  // namespace

int launch_gate_on(cudaStream_t st, ps_state *h, int32_t code, int64_t a, int64_t b, const u64 *flag) {
    const int64_t work = h->W * (h->w >> 1);
    const int grid = blocks_for(work);
    if (h->n == 0 || work == 0) return OK;
    switch (code) {
    case OP_H: gate1_kernel<OP_H><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, nullptr); break;
    case OP_S: gate1_kernel<OP_S><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, nullptr); break;
    case OP_X: gate1_kernel<OP_X><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, nullptr); break;
    case OP_Y: gate1_kernel<OP_Y><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, nullptr); break;
    case OP_Z: gate1_kernel<OP_Z><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, nullptr); break;
    case OP_H_IF: gate1_kernel<OP_H_IF><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, flag); break;
    case OP_S_IF: gate1_kernel<OP_S_IF><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, flag); break;
    case OP_CX: gate2_kernel<OP_CX><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, b); break;
    case OP_CZ: gate2_kernel<OP_CZ><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, b); break;
    default: return fail(E_ARG, "unknown gate code " + std::to_string(code));
    }
    PS_CUDA(cudaGetLastError());
    return OK;
}

int launch_gate(ps_state *h, int32_t code, int64_t a, int64_t b, const u64 *flag) {
    return launch_gate_on(h->stream, h, code, a, b, flag);
}

int launch_channel_rp(cudaStream_t st, ps_state *h, int64_t a, int64_t b, const uint64_t *dev_thr, int count,
                      uint32_t event_off, const RunParams *rp, u64 *masks) {
    channel_sample_kernel<<<blocks_for(h->w), 256, 0, st>>>(masks, h->w, (uint64_t)h->seed, event_off, (uint64_t)h->word_base, rp, count,
                                                             dev_thr);
    PS_CUDA(cudaGetLastError());
    const int64_t work = h->W * (h->w >> 1);
    if (h->n > 0 && work > 0) {
        sign_flip_kernel<<<blocks_for(work), 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, masks, masks + h->w);
        if (count == 15)
            sign_flip_kernel<<<blocks_for(work), 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, b,
                                                                masks + 2 * h->w, masks + 3 * h->w);
    }
    PS_CUDA(cudaGetLastError());
    return OK;
}

int launch_channel_apply(cudaStream_t st, ps_state *h, int64_t a, int64_t b, const uint64_t *dev_thr, int count,
                         const uint32_t *dev_surv, ChannelEst est, uint32_t event_off, const RunParams *rp) {
    if (h->n == 0 || h->w == 0) return OK;
    const dim3 grid((unsigned)((h->w + 7) / 8), (unsigned)((h->W + 63) / 64));
    if (count == 15)
        channel_apply_kernel<1><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, b, event_off, rp, dev_thr,
                                                      count, dev_surv, est);
    else
        channel_apply_kernel<0><<<grid, 256, 0, st>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, 0, event_off, rp, dev_thr,
                                                      count, dev_surv, est);
    PS_CUDA(cudaGetLastError());
    return OK;
}

int check_channel_probs(const float *p, int count) {
    for (int k = 0; k < count; ++k)
        if (!std::isfinite(p[k]) || p[k] < 0.0f || p[k] > 1.0f)
            return fail(E_ARG, "channel probability " + std::to_string(k) + " is not a number in [0, 1]");
    return OK;
}

void channel_thresholds(const float *p, int count, uint64_t *thr) {
    double cum = 0.0;
    for (int k = 0; k < count; ++k) {
        cum += (double)p[k];
        if (!(cum > 0.0))
            thr[k] = 0;
        else if (cum >= 1.0)
            thr[k] = (uint64_t)1 << 32;
        else
            thr[k] = (uint64_t)std::floor(cum * 4294967296.0);
    }
    thr[count] = channel_surv64(thr[count - 1]);
}

int launch_pauli_channel(ps_state *h, int64_t a, int64_t b, const uint64_t *thr, int count) {
    const uint64_t event = h->events++;
    uint64_t *dthr = nullptr;
    PS_CUDA(cudaMallocAsync(&dthr, 16 * sizeof(uint64_t), h->stream));
    PS_CUDA(cudaMemcpyAsync(dthr, thr, (size_t)(count + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
    channel_sample_kernel<<<blocks_for(h->w), 256, 0, h->stream>>>(h->mask_buf, h->w, (uint64_t)h->seed, event, (uint64_t)h->word_base,
                                                                    nullptr, count, dthr);
    PS_CUDA(cudaGetLastError());
    const int64_t work = h->W * (h->w >> 1);
    if (h->n > 0 && work > 0) {
        sign_flip_kernel<<<blocks_for(work), 256, 0, h->stream>>>(h->X, h->Z, h->R, h->n, h->W, h->w, a, h->mask_buf,
                                                                  h->mask_buf + h->w);
        if (count == 15)
            sign_flip_kernel<<<blocks_for(work), 256, 0, h->stream>>>(h->X, h->Z, h->R, h->n, h->W, h->w, b,
                                                                      h->mask_buf + 2 * h->w, h->mask_buf + 3 * h->w);
    }
    PS_CUDA(cudaGetLastError());
    PS_CUDA(cudaFreeAsync(dthr, h->stream));
    return OK;
}

}  // namespace ps

// ---------------------------------------------------------------------------
// Pauli channel without device allocation.
//
// Some callers cannot allocate device memory while they run: a host that
// reserved the whole device for its own pool before starting, code that runs
// under a memory-budget sandbox, or a caller that must not synchronise the
// device (cudaMalloc / cudaFree can).  ps_pauli_channel_1 asks the stream
// allocator for its threshold table on every call; this variant keeps that
// table and the per-word outcome masks in one fixed array linked into the
// library instead; the thresholds reach it as kernel arguments.
//
// Limit: at most NOALLOC_MAX_WORDS shot-words per state (524,288 shots).  The
// array is a module-scope __device__ variable, so every GPU that loads the
// library holds it (258 KiB) until the process exits.  All calls share it and
// it keeps the last call's contents: every word a call reads is written by
// that same call first (thresholds, then all 4*w mask words), so nothing has
// to be cleared.  Calls whose work overlaps on the GPU (different streams)
// race on the array; calls on one stream are ordered.
namespace ps {

namespace {
constexpr int64_t NOALLOC_MAX_WORDS = 8192;
constexpr int NOALLOC_THR = 16;  // threshold slots in front of the masks

static __device__ __align__(256) u64 g_noalloc_scratch[NOALLOC_THR + 4 * NOALLOC_MAX_WORDS];

__global__ void noalloc_set_thresholds(uint64_t *thr, uint64_t t0, uint64_t t1, uint64_t t2, uint64_t s64) {
    thr[0] = t0;
    thr[1] = t1;
    thr[2] = t2;
    thr[3] = s64;
}

// Id of the current CUDA context, 0 when it cannot be had (no context yet,
// or a driver without cuCtxGetId).  The driver calls are fetched through the
// runtime, so the library does not link the driver library itself.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(p);
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the array, kept per device together with the id of the
// context it was looked up in: a context torn down and created again (after
// cudaDeviceReset) loads the module again, possibly elsewhere, and gets a
// new id, so the address is looked up again.  Without an id the address is
// looked up on every call.  A lookup should not happen during stream
// capture.
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {nullptr};
unsigned long long g_noalloc_ctx[64] = {0};

int noalloc_scratch(int dev, u64 **out) {
    if (dev < 0 || dev >= 64) return fail(E_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_noalloc_ptr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = p;
        g_noalloc_ctx[dev] = current_context_id();  // the lookup made the context current if it was not
    }
    *out = static_cast<u64 *>(g_noalloc_ptr[dev]);
    return OK;
}
}  // namespace

int launch_pauli_channel_noalloc(ps_state *h, int64_t q, const uint64_t *thr3) {
    if (h->w > NOALLOC_MAX_WORDS)
        return fail(E_ARG, "batch_size " + std::to_string(h->S) + " exceeds the allocation-free limit of " +
                               std::to_string(NOALLOC_MAX_WORDS * 64) + " shots");
    int dev = 0;
    PS_CUDA(cudaGetDevice(&dev));
    if (dev != h->device) return fail(E_STATE, "the handle belongs to another device than the current one");
    u64 *scratch = nullptr;
    int rc = noalloc_scratch(dev, &scratch);
    if (rc != OK) return rc;
    uint64_t *thr = reinterpret_cast<uint64_t *>(scratch);
    u64 *masks = scratch + NOALLOC_THR;
    const uint64_t event = h->events++;
    // Thresholds travel as kernel arguments (no host copy, no allocation).
    noalloc_set_thresholds<<<1, 1, 0, h->stream>>>(thr, thr3[0], thr3[1], thr3[2], thr3[3]);
    channel_sample_kernel<<<blocks_for(h->w), 256, 0, h->stream>>>(masks, h->w, (uint64_t)h->seed, event, (uint64_t)h->word_base,
                                                                        nullptr, 3, thr);
    PS_CUDA(cudaGetLastError());
    const int64_t work = h->W * (h->w >> 1);
    if (h->n > 0 && work > 0)
        sign_flip_kernel<<<blocks_for(work), 256, 0, h->stream>>>(h->X, h->Z, h->R, h->n, h->W, h->w, q, masks,
                                                                  masks + h->w);
    PS_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace ps
