// ps_state.cu -- device tableau lifetime, initialisation, reference-layout
// import/export, checksum and measurement-record storage.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <set>
#include <vector>

#include "ps_internal.h"

namespace ps {

namespace {

// InitTableauToZeroStateFunctor (MiscFunctors.hpp:8-28): x(i,j)=[i==j],
// z(i,j)=[i-n==j], r(i)=[i==2n], for every shot (all 64 bits of a word).
__global__ void init_zero_kernel(u64 *__restrict__ X, u64 *__restrict__ Z, u64 *__restrict__ R, int64_t n, int64_t W,
                                 int64_t w) {
    const int64_t cells = W * n * w;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < cells; idx += stride) {
        const int64_t col = idx / w;  // row*n + j
        const int64_t i = col / n, j = col - i * n;
        X[idx] = (i == j) ? ~0ull : 0ull;
        Z[idx] = (i - n == j) ? ~0ull : 0ull;
    }
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < W * w; idx += stride) {
        const int64_t i = idx / w;
        R[idx] = (i == 2 * n) ? ~0ull : 0ull;
    }
}

// Host int32 [shots][W][n] chunk -> packed bits of words [k0, k0+chunk).
// One thread per int32 cell (coalesced reads); set bits are OR-ed in.
__global__ void pack_kernel(const int32_t *__restrict__ hx, const int32_t *__restrict__ hz,
                            const int32_t *__restrict__ hr, u64 *X, u64 *Z, u64 *R, int64_t n, int64_t W, int64_t w,
                            int64_t shot0, int64_t nshots) {
    const int64_t cells = nshots * W * n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < cells; idx += stride) {
        const int64_t s = idx / (W * n);
        const int64_t rem = idx - s * W * n;
        const int64_t gs = shot0 + s;
        const int64_t word = gs >> 6;
        const u64 bit = 1ull << (gs & 63);
        const int64_t off = rem * w + word;  // (i*n + j)*w + word
        if (hx[idx]) atomicOr(&X[off], bit);
        if (hz[idx]) atomicOr(&Z[off], bit);
    }
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nshots * W; idx += stride) {
        const int64_t s = idx / W, i = idx - s * W;
        const int64_t gs = shot0 + s;
        if (hr[idx]) atomicOr(&R[i * w + (gs >> 6)], 1ull << (gs & 63));
    }
}

__global__ void unpack_kernel(int32_t *__restrict__ hx, int32_t *__restrict__ hz, int32_t *__restrict__ hr,
                              const u64 *__restrict__ X, const u64 *__restrict__ Z, const u64 *__restrict__ R,
                              int64_t n, int64_t W, int64_t w, int64_t shot0, int64_t nshots) {
    const int64_t cells = nshots * W * n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < cells; idx += stride) {
        const int64_t s = idx / (W * n);
        const int64_t rem = idx - s * W * n;
        const int64_t gs = shot0 + s;
        const int64_t off = rem * w + (gs >> 6);
        hx[idx] = (int32_t)((X[off] >> (gs & 63)) & 1ull);
        hz[idx] = (int32_t)((Z[off] >> (gs & 63)) & 1ull);
    }
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nshots * W; idx += stride) {
        const int64_t s = idx / W, i = idx - s * W;
        const int64_t gs = shot0 + s;
        hr[idx] = (int32_t)((R[i * w + (gs >> 6)] >> (gs & 63)) & 1ull);
    }
}

__device__ __forceinline__ u64 range_mask(int64_t word, int64_t s0, int64_t s1) {
    const int64_t lo = word * 64, hi = lo + 64;
    const int64_t a = max(lo, s0), b = min(hi, s1);
    if (a >= b) return 0ull;
    const int64_t len = b - a;
    const u64 m = len == 64 ? ~0ull : ((1ull << len) - 1ull);
    return m << (a - lo);
}

// CheckSumFunctor (MiscFunctors.hpp:30-50): popcount of x, z and r bits of
// shots [s0, s1).
__global__ void checksum_kernel(const u64 *__restrict__ X, const u64 *__restrict__ Z, const u64 *__restrict__ R,
                                int64_t n, int64_t W, int64_t w, int64_t s0, int64_t s1,
                                unsigned long long *__restrict__ out) {
    unsigned long long acc = 0;
    const int64_t cells = W * n * w;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < cells; idx += stride) {
        const u64 m = range_mask(idx % w, s0, s1);
        acc += __popcll(X[idx] & m) + __popcll(Z[idx] & m);
    }
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < W * w; idx += stride)
        acc += __popcll(R[idx] & range_mask(idx % w, s0, s1));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

int grid_for(int64_t work, int threads = 256) {
    int64_t blocks = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(blocks, 152 * 16));
}

}  // namespace

int allow_max_smem(const void *kernel) {
    static std::mutex mu;
    static std::set<std::pair<const void *, int>> done;
    int dev = 0;
    PS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({kernel, dev})) return OK;
    int optin = 0;
    PS_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    PS_CUDA(cudaFuncGetAttributes(&fa, kernel));
    const int dyn = optin - (int)fa.sharedSizeBytes;  // static shared memory counts against the limit
    PS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
    done.insert({kernel, dev});
    return OK;
}

int dev_alloc(ps_state *h, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    if (h->pool) {
        if (!h->pool->alloc(p, bytes)) return fail(E_NOMEM, "device pool exhausted (" + std::to_string(bytes >> 20) + " MiB requested)");
        return OK;
    }
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(E_NOMEM, "device allocation failed (" + std::to_string(bytes >> 20) + " MiB): " +
                                 cudaGetErrorString(e));
    }
    return OK;
}

void dev_free(ps_state *h, void *p) {
    if (!p) return;
    if (h->pool)
        h->pool->release(p);
    else
        cudaFree(p);
}

int state_alloc(ps_state *h, int64_t n, int64_t S, int64_t seed, DevPool *pool, bool signs_only) {
    h->n = n;
    h->signs_only = signs_only;
    h->S = S;
    h->W = 2 * n + 1;
    h->pool = pool;
    int64_t w = (S + 63) / 64;
    w = (w + 1) & ~int64_t(1);  // even: every column starts 16-byte aligned
    if (w == 0) w = 2;
    h->w = w;
    h->seed = seed >= 0 ? seed : 213434232223LL;  // CliffordState.hpp:130-138
    PS_CUDA(cudaGetDevice(&h->device));
    PS_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    const size_t plane = (size_t)h->W * (size_t)(n > 0 ? n : 1) * (size_t)w * sizeof(u64);
    void *px = nullptr, *pz = nullptr, *pr = nullptr;
    if ((!signs_only && (dev_alloc(h, &px, plane) != OK || dev_alloc(h, &pz, plane) != OK)) ||
        dev_alloc(h, &pr, (size_t)h->W * w * sizeof(u64)) != OK) {
        dev_free(h, px);
        dev_free(h, pz);
        return fail(E_NOMEM, "device allocation of the tableau failed (" + std::to_string(3 * plane >> 20) + " MiB)");
    }
    h->X = (u64 *)px;
    h->Z = (u64 *)pz;
    h->R = (u64 *)pr;
    void *pf = nullptr, *pm = nullptr;
    if (dev_alloc(h, &pf, (size_t)w * sizeof(u64)) != OK) return E_NOMEM;
    h->forced_buf = (u64 *)pf;
    if (dev_alloc(h, &pm, (size_t)4 * w * sizeof(u64)) != OK) return E_NOMEM;
    h->mask_buf = (u64 *)pm;
    h->arena.words = (size_t)w;
    return OK;
}

// Bytes state_alloc takes for a state of n qubits and S shots.
size_t state_bytes(int64_t n, int64_t S, bool signs_only) {
    int64_t w = (S + 63) / 64;
    w = (w + 1) & ~int64_t(1);
    if (w == 0) w = 2;
    const size_t W = 2 * (size_t)n + 1;
    return (signs_only ? 0 : 2 * W * (size_t)(n > 0 ? n : 1) * (size_t)w * 8) + W * (size_t)w * 8 + 5 * (size_t)w * 8;
}

void state_free(ps_state *h) {
    if (h->stream) cudaStreamSynchronize(h->stream);
    dev_free(h, h->X);
    dev_free(h, h->Z);
    dev_free(h, h->R);
    dev_free(h, h->forced_buf);
    dev_free(h, h->mask_buf);
    dev_free(h, h->meas_buf);
    for (u64 *c : h->arena.chunks) dev_free(h, c);
    for (u64 *c : h->arena.blocks) dev_free(h, c);
    h->arena.chunks.clear();
    h->arena.blocks.clear();
    if (h->stream) cudaStreamDestroy(h->stream);
    h->X = h->Z = h->R = nullptr;
    h->forced_buf = h->mask_buf = nullptr;
    h->meas_buf = nullptr;
}

int launch_init_zero_on(cudaStream_t stream, ps_state *h) {
    if (h->n == 0) return OK;
    init_zero_kernel<<<grid_for(h->W * h->n * h->w), 256, 0, stream>>>(h->X, h->Z, h->R, h->n, h->W, h->w);
    PS_CUDA(cudaGetLastError());
    return OK;
}

int launch_init_zero(ps_state *h) { return launch_init_zero_on(h->stream, h); }

int record_new(ps_state *h, int64_t q, int64_t *id) {
    RecordArena &a = h->arena;
    if (a.chunks.empty() || a.used_in_last == a.per_chunk) {
        void *chunk = nullptr;
        if (dev_alloc(h, &chunk, a.per_chunk * 2 * a.words * sizeof(u64)) != OK)
            return fail(E_NOMEM, "device allocation of measurement records failed");
        a.chunks.push_back((u64 *)chunk);
        a.used_in_last = 0;
    }
    Record rec;
    rec.qubit = q;
    rec.res = a.chunks.back() + a.used_in_last * 2 * a.words;
    rec.det = rec.res + a.words;
    a.used_in_last++;
    PS_CUDA(cudaMemsetAsync(rec.res, 0, 2 * a.words * sizeof(u64), h->stream));
    h->recs.push_back(std::move(rec));
    *id = (int64_t)h->recs.size() - 1;
    return OK;
}

int record_block(ps_state *h, const std::vector<int64_t> &qubits, std::vector<int64_t> &ids, u64 **res_block,
                 u64 **det_block) {
    const size_t nm = qubits.size(), wds = (size_t)h->w;
    ids.clear();
    *res_block = *det_block = nullptr;
    if (nm == 0) return OK;
    void *pblk = nullptr;
    if (dev_alloc(h, &pblk, 2 * nm * wds * sizeof(u64)) != OK)
        return fail(E_NOMEM, "device allocation of measurement records failed");
    u64 *blk = (u64 *)pblk;
    PS_CUDA(cudaMemsetAsync(blk, 0, 2 * nm * wds * sizeof(u64), h->stream));
    // The state owns the block (freed with the state), like its other records.
    h->arena.blocks.push_back(blk);
    *res_block = blk;
    *det_block = blk + nm * wds;
    for (size_t k = 0; k < nm; ++k) {
        Record rec;
        rec.qubit = qubits[k];
        rec.res = blk + k * wds;
        rec.det = blk + (nm + k) * wds;
        h->recs.push_back(std::move(rec));
        ids.push_back((int64_t)h->recs.size() - 1);
    }
    return OK;
}

int record_fetch(ps_state *h, int64_t id) {
    Record &rec = h->recs[(size_t)id];
    if (rec.host_valid) return OK;
    rec.host_res.resize((size_t)h->w);
    rec.host_det.resize((size_t)h->w);
    PS_CUDA(cudaMemcpyAsync(rec.host_res.data(), rec.res, (size_t)h->w * 8, cudaMemcpyDeviceToHost, h->stream));
    PS_CUDA(cudaMemcpyAsync(rec.host_det.data(), rec.det, (size_t)h->w * 8, cudaMemcpyDeviceToHost, h->stream));
    PS_CUDA(cudaStreamSynchronize(h->stream));
    rec.host_valid = true;
    return OK;
}

int upload_forced(ps_state *h, const uint8_t *forced, const u64 **dev) {
    if (!forced) {
        *dev = nullptr;
        return OK;
    }
    std::vector<u64> tmp((size_t)h->w, 0ull);
    std::memcpy(tmp.data(), forced, (size_t)(h->S + 7) / 8);
    if (h->S % 8) {  // clear the unused high bits of the last byte
        uint8_t *b = reinterpret_cast<uint8_t *>(tmp.data());
        b[(h->S - 1) / 8] &= (uint8_t)((1u << (h->S % 8)) - 1u);
    }
    PS_CUDA(cudaMemcpyAsync(h->forced_buf, tmp.data(), (size_t)h->w * 8, cudaMemcpyHostToDevice, h->stream));
    PS_CUDA(cudaStreamSynchronize(h->stream));  // tmp leaves scope
    *dev = h->forced_buf;
    return OK;
}

// Chunk of shots converted per staging round (bounded device staging).
static int64_t shots_per_chunk(const ps_state *h) {
    const int64_t cell_bytes = (h->W * h->n + h->W) * 4 * 3;
    int64_t words = std::max<int64_t>(1, (int64_t(256) << 20) / std::max<int64_t>(1, cell_bytes * 64));
    return words * 64;
}

int pack_from_host(ps_state *h, const int32_t *x, const int32_t *z, const int32_t *r) {
    const size_t plane = (size_t)h->W * h->n * h->w * sizeof(u64);
    PS_CUDA(cudaMemsetAsync(h->X, 0, plane, h->stream));
    PS_CUDA(cudaMemsetAsync(h->Z, 0, plane, h->stream));
    PS_CUDA(cudaMemsetAsync(h->R, 0, (size_t)h->W * h->w * sizeof(u64), h->stream));
    if (h->n == 0 || h->S == 0) return OK;
    const int64_t chunk = std::min<int64_t>(shots_per_chunk(h), h->S);
    const size_t cells = (size_t)chunk * h->W * h->n;
    int32_t *dx = nullptr, *dz = nullptr, *dr = nullptr;
    PS_CUDA(cudaMalloc(&dx, cells * 4));
    PS_CUDA(cudaMalloc(&dz, cells * 4));
    PS_CUDA(cudaMalloc(&dr, (size_t)chunk * h->W * 4));
    int rc = OK;
    for (int64_t s0 = 0; s0 < h->S && rc == OK; s0 += chunk) {
        const int64_t ns = std::min(chunk, h->S - s0);
        const size_t c = (size_t)ns * h->W * h->n;
        if (cudaMemcpyAsync(dx, x + (size_t)s0 * h->W * h->n, c * 4, cudaMemcpyHostToDevice, h->stream) ||
            cudaMemcpyAsync(dz, z + (size_t)s0 * h->W * h->n, c * 4, cudaMemcpyHostToDevice, h->stream) ||
            cudaMemcpyAsync(dr, r + (size_t)s0 * h->W, (size_t)ns * h->W * 4, cudaMemcpyHostToDevice, h->stream)) {
            rc = cuda_fail(cudaGetLastError(), "cudaMemcpyAsync (host_to_device)");
            break;
        }
        pack_kernel<<<grid_for((int64_t)c), 256, 0, h->stream>>>(dx, dz, dr, h->X, h->Z, h->R, h->n, h->W, h->w, s0, ns);
        cudaError_t e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "pack_kernel");
    }
    cudaFree(dx);
    cudaFree(dz);
    cudaFree(dr);
    return rc;
}

int unpack_to_host(ps_state *h, int32_t *x, int32_t *z, int32_t *r) {
    if (h->n == 0 || h->S == 0) return OK;
    const int64_t chunk = std::min<int64_t>(shots_per_chunk(h), h->S);
    const size_t cells = (size_t)chunk * h->W * h->n;
    int32_t *dx = nullptr, *dz = nullptr, *dr = nullptr;
    PS_CUDA(cudaMalloc(&dx, cells * 4));
    PS_CUDA(cudaMalloc(&dz, cells * 4));
    PS_CUDA(cudaMalloc(&dr, (size_t)chunk * h->W * 4));
    int rc = OK;
    for (int64_t s0 = 0; s0 < h->S && rc == OK; s0 += chunk) {
        const int64_t ns = std::min(chunk, h->S - s0);
        const size_t c = (size_t)ns * h->W * h->n;
        unpack_kernel<<<grid_for((int64_t)c), 256, 0, h->stream>>>(dx, dz, dr, h->X, h->Z, h->R, h->n, h->W, h->w, s0, ns);
        if (cudaMemcpyAsync(x + (size_t)s0 * h->W * h->n, dx, c * 4, cudaMemcpyDeviceToHost, h->stream) ||
            cudaMemcpyAsync(z + (size_t)s0 * h->W * h->n, dz, c * 4, cudaMemcpyDeviceToHost, h->stream) ||
            cudaMemcpyAsync(r + (size_t)s0 * h->W, dr, (size_t)ns * h->W * 4, cudaMemcpyDeviceToHost, h->stream)) {
            rc = cuda_fail(cudaGetLastError(), "cudaMemcpyAsync (device_to_host)");
            break;
        }
        cudaError_t e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "unpack_kernel");
    }
    cudaFree(dx);
    cudaFree(dz);
    cudaFree(dr);
    return rc;
}

int checksum(ps_state *h, int64_t s0, int64_t s1, int64_t *out) {
    unsigned long long *d = nullptr, v = 0;
    PS_CUDA(cudaMallocAsync(&d, sizeof(unsigned long long), h->stream));
    PS_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), h->stream));
    if (h->n > 0 && s1 > s0)
        checksum_kernel<<<grid_for(h->W * h->n * h->w), 256, 0, h->stream>>>(h->X, h->Z, h->R, h->n, h->W, h->w, s0,
                                                                            s1, d);
    PS_CUDA(cudaGetLastError());
    PS_CUDA(cudaMemcpyAsync(&v, d, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    PS_CUDA(cudaFreeAsync(d, h->stream));
    PS_CUDA(cudaStreamSynchronize(h->stream));
    *out = (int64_t)v;
    return OK;
}

}  // namespace ps
