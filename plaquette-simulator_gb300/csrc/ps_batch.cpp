// ps_batch.cpp -- many sampling jobs at once: batches (one CUDA graph launch
// whose branches are the jobs) and the serving loop (continuous admission of
// jobs against an HBM budget, one stream per active job).  Neither has a
// counterpart in the reference, which runs one CliffordState at a time
// (CliffordState.hpp:97-139); every job here is a compiled circuit on its own
// state and gives the same records as when it runs alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <numeric>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/plaquette_gpu.h"
#include "ps_frame_dev.h"
#include "ps_internal.h"
#include "ps_segment.cuh"

#define TRY(expr)                     \
    do {                              \
        const int _rc = (expr);       \
        if (_rc != ps::OK) return _rc; \
    } while (0)

namespace ps {

// ------------------------------------------------------------ DevPool
void DevPool::reset(void *region, size_t bytes) {
    std::lock_guard<std::mutex> lk(mu);
    base = static_cast<char *>(region);
    cap = bytes;
    used = peak = 0;
    free_.clear();
    taken.clear();
    if (bytes) free_[0] = bytes;
}

bool DevPool::alloc(void **p, size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    std::lock_guard<std::mutex> lk(mu);
    auto best = free_.end();
    for (auto it = free_.begin(); it != free_.end(); ++it)
        if (it->second >= bytes && (best == free_.end() || it->second < best->second)) best = it;
    if (best == free_.end()) return false;
    const size_t off = best->first, sz = best->second;
    free_.erase(best);
    if (sz > bytes) free_[off + bytes] = sz - bytes;
    taken[off] = bytes;
    used += bytes;
    peak = std::max(peak, used);
    *p = base + off;
    return true;
}

void DevPool::release(void *p) {
    std::lock_guard<std::mutex> lk(mu);
    const size_t off = (size_t)(static_cast<char *>(p) - base);
    auto t = taken.find(off);
    if (t == taken.end()) return;
    size_t start = off, sz = t->second;
    taken.erase(t);
    used -= sz;
    auto nx = free_.lower_bound(off);
    if (nx != free_.end() && off + sz == nx->first) {
        sz += nx->second;
        nx = free_.erase(nx);
    }
    if (nx != free_.begin()) {
        auto pv = std::prev(nx);
        if (pv->first + pv->second == off) {
            pv->second += sz;
            return;
        }
    }
    free_[start] = sz;
}

namespace {

// Writes each job's run parameters (seed, event base) into its circuit's
// device slot: the root node of a batch graph.
__global__ void batch_params_kernel(RunParams *const *__restrict__ dst, const RunParams *__restrict__ src, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) *dst[i] = src[i];
}

bool is_meas_code(int32_t c) { return c == OP_M || c == OP_R; }
bool is_channel_code(int32_t c) { return c == OP_PAULI1 || c == OP_PAULI2; }

uint64_t count_gates(const ps_op *ops, uint64_t nops) {
    uint64_t g = 0;
    for (uint64_t i = 0; i < nops; ++i) g += ops[i].code <= OP_R ? 1 : 0;
    return g;
}

// Upper bound of the device bytes a fused job takes: tableau, records, the
// channel-outcome scratch of its largest segment, schedule tables.  Signs
// only (a sampling job of the request loop): the signs, records, the noise
// vectors of the shared-x/z plan (one [shot-word][row] block for each run of
// gates holding a channel) and its tables (a channel's rows taken as at most
// 128 words, the usual case; an allocation beyond the estimate fails as a
// full pool and the job is admitted again later).
size_t job_device_bytes(const ps_job_desc &j, bool signs_only) {
    int64_t w = ((int64_t)j.shots + 63) / 64;
    w = (w + 1) & ~int64_t(1);
    if (w == 0) w = 2;
    size_t nm = 0, nch = 0, seg_ch = 0, max_ch = 0, noisy_runs = 0;
    for (uint64_t i = 0; i < j.nops; ++i) {
        const int32_t c = j.ops[i].code;
        if (is_meas_code(c)) {
            ++nm;
            seg_ch = 0;
        } else if (is_channel_code(c)) {
            ++nch;
            if (seg_ch == 0) ++noisy_runs;
            max_ch = std::max(max_ch, ++seg_ch);
        }
    }
    const size_t W = (size_t)w;
    size_t b = state_bytes((int64_t)j.num_qubits, (int64_t)j.shots, signs_only);
    b += 2 * nm * W * 8;  // records
    if (signs_only) {
        const size_t wp = (2 * (size_t)j.num_qubits + 2) & ~(size_t)1;
        b += noisy_runs * W * wp * 8;                      // noise vectors
        b += nch * (128 * 4 + 32) + (size_t)j.nops * 64;  // channel rows and records, program
    } else {
        b += std::max<size_t>(1, max_ch) * W * (sizeof(NoiseEntry) + 32) + W * 4;  // outcome scratch
    }
    b += 4 * W * 8 + 64;                                             // masks, params
    b += (size_t)j.nops * 128 + nch * 15 * 8 + nm * sizeof(MeasOp);  // schedules
    b += 64 * 256 + (1u << 20);                                      // granules, slack
    return b;
}

// A job runs on a signs-only state when no gate depends on a measurement
// record (its x / z are the same in every shot).
bool signs_only_job(const ps_job_desc &j) {
    for (uint64_t i = 0; i < j.nops; ++i)
        if (j.ops[i].code == OP_H_IF || j.ops[i].code == OP_S_IF) return false;
    return j.num_qubits > 0;
}

int check_job(const ps_job_desc &j, uint64_t index) {
    if (!j.ops && j.nops) return fail(E_ARG, "job " + std::to_string(index) + ": null op table");
    if (j.num_qubits == 0 || j.shots == 0) return fail(E_ARG, "job " + std::to_string(index) + ": empty job");
    if (j.num_qubits > 2048) return fail(E_ARG, "job " + std::to_string(index) + ": more than 2048 qubits");
    return OK;
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace
}  // namespace ps

using namespace ps;

// ================================================================ batches
struct ps_batch {
    ps_batch_options opts{};
    ps_batch_stats stats{};
    int device = 0;
    std::vector<ps_state *> states;
    std::vector<ps_circuit *> circs;
    std::vector<size_t> order;  // launch order: most shot-gates first
    cudaStream_t stream = nullptr;
    std::vector<cudaStream_t> branches;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> joins;
    static constexpr int RING = 4;
    RunParams *h_vals[RING] = {};
    cudaEvent_t copied[RING] = {};
    int ring_pos = 0;
    RunParams *d_vals = nullptr;
    RunParams **d_dst = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // Jobs that run the shared-x/z plan share one job table: each of its
    // kernels (noise vectors, signs, x / z broadcast) is one launch for all
    // of them.  The others run their own plans on branches.
    std::vector<size_t> table_jobs;  // job indices, in table order
    std::vector<char> in_table;      // [job]
    ps::FrameTable table;
    std::vector<void *> table_mem;
    cudaStream_t side = nullptr;
    cudaEvent_t tfork = nullptr, tjoin = nullptr;
    int frame_warps = 8, bcast_ctas = 1;
};

namespace ps {
namespace {

// Root scatter node, then the job table's kernels on the main stream and
// every other job on its own branch, joined back.
int enqueue_batch(ps_batch *b) {
    const int nj = (int)b->circs.size();
    batch_params_kernel<<<1, 256, 0, b->stream>>>(b->d_dst, b->d_vals, nj);
    PS_CUDA(cudaGetLastError());
    PS_CUDA(cudaEventRecord(b->fork, b->stream));
    if (!b->table_jobs.empty())
        TRY(frame_table_enqueue(b->table, b->stream, b->side, b->tfork, b->tjoin, b->frame_warps, b->bcast_ctas));
    for (size_t k = 0; k < b->order.size(); ++k) {
        const size_t j = b->order[k];
        if (b->in_table[j]) continue;
        PS_CUDA(cudaStreamWaitEvent(b->branches[k], b->fork, 0));
        TRY(circuit_enqueue(b->circs[j], b->branches[k], true));
        PS_CUDA(cudaEventRecord(b->joins[k], b->branches[k]));
        PS_CUDA(cudaStreamWaitEvent(b->stream, b->joins[k], 0));
    }
    return OK;
}

}  // namespace
}  // namespace ps

extern "C" {

ps_status ps_batch_destroy(ps_batch *b);

ps_status ps_batch_create(const ps_job_desc *jobs, uint64_t njobs, const ps_batch_options *opts, ps_batch **out) {
    ps_enter(__func__, __LINE__);
    if (!out || (!jobs && njobs)) return fail(E_ARG, "null argument");
    *out = nullptr;
    if (njobs == 0) return fail(E_ARG, "empty batch");
    for (uint64_t j = 0; j < njobs; ++j) TRY(check_job(jobs[j], j));
    auto *b = new ps_batch;
    if (opts) b->opts = *opts;
    auto bail = [&](int rc) {
        const std::string msg = ps_last_error();
        ps_batch_destroy(b);
        set_error(msg);  // keep the failing call's message
        return rc;
    };
    PS_CUDA(cudaGetDevice(&b->device));
    const auto t0 = std::chrono::steady_clock::now();
    b->states.assign(njobs, nullptr);
    b->circs.assign(njobs, nullptr);
    // Jobs compile in parallel on the host (schedules, bank-group search).
    std::vector<int> rcs(njobs, OK);
    std::vector<std::string> errs(njobs);
    {
        std::atomic<uint64_t> next{0};
        const unsigned nt = std::max(1u, std::min<unsigned>(16, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < std::min<uint64_t>(nt, njobs); ++t)
            pool.emplace_back([&] {
                cudaSetDevice(b->device);
                for (uint64_t j = next++; j < njobs; j = next++) {
                    const ps_job_desc &jd = jobs[j];
                    int rc = ps_create(jd.num_qubits, jd.shots, jd.seed, 1, &b->states[j]);
                    if (rc == OK) {
                        ps_circuit_options co{};
                        co.mode = PS_MODE_FUSED;
                        co.use_graph = 0;
                        rc = ps_circuit_compile(b->states[j], jd.ops, jd.nops, jd.params, jd.nparams, &co, &b->circs[j]);
                    }
                    if (rc != OK) errs[j] = "job " + std::to_string(j) + ": " + ps_last_error();
                    rcs[j] = rc;
                }
            });
        for (auto &t : pool) t.join();
    }
    for (uint64_t j = 0; j < njobs; ++j)
        if (rcs[j] != OK) {
            fail(rcs[j], errs[j]);
            return bail(rcs[j]);
        }
    b->stats.compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (b->opts.autotune) {  // the per-shot plans (jobs of the table are tuned together below)
        for (uint64_t j = 0; j < njobs; ++j) {
            FrameJobDev fjd{};
            BroadcastJobDev bjd{};
            if (circuit_frame_job(b->circs[j], &fjd, &bjd)) continue;
            double ms = 0.0;
            int rc = ps_circuit_autotune(b->circs[j], nullptr, &ms);
            if (rc != OK) return bail(rc);
            b->stats.tune_ms += ms;
        }
    }
    // ---- stats and launch order
    std::vector<double> work(njobs);
    for (uint64_t j = 0; j < njobs; ++j) {
        ps_circuit_stats cs{};
        ps_circuit_get_stats(b->circs[j], &cs);
        b->stats.shot_gates_per_run += cs.num_gates * jobs[j].shots;
        b->stats.tableau_bytes += state_bytes((int64_t)jobs[j].num_qubits, (int64_t)jobs[j].shots);
        b->stats.launches_per_run += cs.launches_per_run;  // its parameter update stands for the init launch
        work[j] = (double)cs.segment_bytes;
    }
    b->stats.launches_per_run += 1;  // the parameter scatter
    b->stats.num_jobs = njobs;
    b->order.resize(njobs);
    std::iota(b->order.begin(), b->order.end(), size_t(0));
    std::stable_sort(b->order.begin(), b->order.end(), [&](size_t x, size_t y) { return work[x] > work[y]; });

    // ---- the job table of the shared-x/z jobs (largest first)
    b->in_table.assign(njobs, 0);
    {
        std::vector<FrameJobDev> fj;
        std::vector<BroadcastJobDev> bj;
        std::vector<int64_t> cta0{0}, ncta0{0}, chunk0{0};
        for (size_t j : b->order) {
            FrameJobDev job{};
            BroadcastJobDev bjob{};
            if (!circuit_frame_job(b->circs[j], &job, &bjob)) continue;
            b->in_table[j] = 1;
            b->table_jobs.push_back(j);
            fj.push_back(job);
            bj.push_back(bjob);
            cta0.push_back(cta0.back() + job.w);
            ncta0.push_back(ncta0.back() + (int64_t)job.nnv * job.w);
            chunk0.push_back(chunk0.back() + broadcast_chunks(job.n, job.w));
            b->table.smem = std::max(b->table.smem, frame_job_smem(job));
            if (job.nnv > 0) b->table.nsmem = std::max(b->table.nsmem, noise_job_smem(job));
        }
        if (!fj.empty()) {
            auto up = [&](const void *src, size_t bytes, void **dst) -> int {
                if (cudaMalloc(dst, std::max<size_t>(bytes, 16)) != cudaSuccess) return cuda_fail(cudaGetLastError(), "cudaMalloc");
                b->table_mem.push_back(*dst);
                PS_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
                return OK;
            };
            void *p[6] = {};
            const unsigned long long zero[2] = {0ull, 0ull};  // the broadcast's counters
            int rc = up(fj.data(), fj.size() * sizeof(FrameJobDev), &p[0]);
            if (rc == OK) rc = up(zero, sizeof zero, &p[5]);
            if (rc == OK) rc = up(bj.data(), bj.size() * sizeof(BroadcastJobDev), &p[1]);
            if (rc == OK) rc = up(cta0.data(), cta0.size() * sizeof(int64_t), &p[2]);
            if (rc == OK) rc = up(ncta0.data(), ncta0.size() * sizeof(int64_t), &p[3]);
            if (rc == OK) rc = up(chunk0.data(), chunk0.size() * sizeof(int64_t), &p[4]);
            if (rc != OK) return bail(rc);
            b->table.jobs = static_cast<const FrameJobDev *>(p[0]);
            b->table.bjobs = static_cast<const BroadcastJobDev *>(p[1]);
            b->table.cta0 = static_cast<const int64_t *>(p[2]);
            b->table.ncta0 = static_cast<const int64_t *>(p[3]);
            b->table.chunk0 = static_cast<const int64_t *>(p[4]);
            b->table.bctr = static_cast<unsigned long long *>(p[5]);
            b->table.njobs = (int32_t)fj.size();
            b->table.ctas = cta0.back();
            b->table.nctas = ncta0.back();
            b->table.chunks = chunk0.back();
            // the table's launches stand for its jobs' own
            for (size_t j : b->table_jobs) {
                ps_circuit_stats cs{};
                ps_circuit_get_stats(b->circs[j], &cs);
                b->stats.launches_per_run -= cs.launches_per_run;
            }
            b->stats.launches_per_run += 1 + (b->table.nctas > 0 ? 1 : 0) + (b->table.chunks > 0 ? 1 : 0);
        }
        b->stats.table_jobs = fj.size();
    }

    // ---- streams, parameter staging
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
        return bail(cuda_fail(cudaGetLastError(), "stream/event"));
    if (!b->table_jobs.empty() &&
        (cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
         cudaEventCreateWithFlags(&b->tfork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&b->tjoin, cudaEventDisableTiming) != cudaSuccess))
        return bail(cuda_fail(cudaGetLastError(), "stream/event"));
    b->branches.assign(njobs, nullptr);
    b->joins.assign(njobs, nullptr);
    for (uint64_t k = 0; k < njobs; ++k)
        if (cudaStreamCreateWithFlags(&b->branches[k], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming) != cudaSuccess)
            return bail(cuda_fail(cudaGetLastError(), "stream/event"));
    for (int r = 0; r < ps_batch::RING; ++r) {
        if (cudaMallocHost(&b->h_vals[r], njobs * sizeof(RunParams)) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->copied[r], cudaEventDisableTiming) != cudaSuccess)
            return bail(cuda_fail(cudaGetLastError(), "pinned staging"));
    }
    if (cudaMalloc(&b->d_vals, njobs * sizeof(RunParams)) != cudaSuccess ||
        cudaMalloc(&b->d_dst, njobs * sizeof(RunParams *)) != cudaSuccess)
        return bail(cuda_fail(cudaGetLastError(), "cudaMalloc"));
    {
        std::vector<RunParams *> dst(njobs);
        for (uint64_t j = 0; j < njobs; ++j) dst[j] = circuit_params_dev(b->circs[j]);
        if (cudaMemcpy(b->d_dst, dst.data(), njobs * sizeof(RunParams *), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(cuda_fail(cudaGetLastError(), "cudaMemcpy"));
    }
    // ---- the table's knobs, timed on the table itself
    if (b->opts.autotune && !b->table_jobs.empty()) {
        const auto tt = std::chrono::steady_clock::now();
        std::vector<RunParams> cur(njobs);
        for (uint64_t j = 0; j < njobs; ++j) cur[j] = circuit_current_params(b->circs[j]);
        if (cudaMemcpy(b->d_vals, cur.data(), njobs * sizeof(RunParams), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(cuda_fail(cudaGetLastError(), "cudaMemcpy"));
        batch_params_kernel<<<1, 256, 0, b->stream>>>(b->d_dst, b->d_vals, (int)njobs);
        int rc = frame_table_tune(b->table, b->stream, b->side, b->tfork, b->tjoin, &b->frame_warps, &b->bcast_ctas,
                                  nullptr);
        if (rc != OK) return bail(rc);
        b->stats.tune_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tt).count();
    }
    b->stats.frame_warps = b->frame_warps;
    b->stats.bcast_ctas = b->bcast_ctas;
    // ---- one graph for the whole batch
    if (b->opts.use_graph) {
        cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
        int rc = e == cudaSuccess ? enqueue_batch(b) : cuda_fail(e, "cudaStreamBeginCapture");
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        if (rc != OK) {
            if (g) cudaGraphDestroy(g);
            return bail(rc);
        }
        if (e2 != cudaSuccess) return bail(cuda_fail(e2, "cudaStreamEndCapture"));
        b->graph = g;
        e = cudaGraphInstantiateWithFlags(&b->exec, g, cudaGraphInstantiateFlagUseNodePriority);
        if (e != cudaSuccess) return bail(cuda_fail(e, "cudaGraphInstantiate"));
    }
    *out = b;
    return OK;
}

ps_status ps_batch_run(ps_batch *b) {
    ps_enter(__func__, __LINE__);
    if (!b) return fail(E_ARG, "null batch");
    NvtxRange range("ps batch run");
    const int slot = b->ring_pos;
    b->ring_pos = (b->ring_pos + 1) % ps_batch::RING;
    PS_CUDA(cudaEventSynchronize(b->copied[slot]));  // the slot's previous copy has been read
    RunParams *vals = b->h_vals[slot];
    for (size_t j = 0; j < b->circs.size(); ++j) vals[j] = circuit_begin_run(b->circs[j], true);
    PS_CUDA(cudaMemcpyAsync(b->d_vals, vals, b->circs.size() * sizeof(RunParams), cudaMemcpyHostToDevice, b->stream));
    PS_CUDA(cudaEventRecord(b->copied[slot], b->stream));
    if (b->exec) {
        PS_CUDA(cudaGraphLaunch(b->exec, b->stream));
        return OK;
    }
    return enqueue_batch(b);
}

ps_status ps_batch_synchronize(ps_batch *b) {
    ps_enter(__func__, __LINE__);
    if (!b) return fail(E_ARG, "null batch");
    PS_CUDA(cudaStreamSynchronize(b->stream));
    return OK;
}

ps_status ps_batch_get_stream(const ps_batch *b, void **stream) {
    ps_enter(__func__, __LINE__);
    if (!b || !stream) return fail(E_ARG, "null argument");
    *stream = (void *)b->stream;
    return OK;
}

ps_status ps_batch_job(const ps_batch *b, uint64_t j, ps_circuit **circuit, ps_state **state) {
    ps_enter(__func__, __LINE__);
    if (!b) return fail(E_ARG, "null batch");
    if (j >= b->circs.size()) return fail(E_RANGE, "job index out of range");
    if (circuit) *circuit = b->circs[j];
    if (state) *state = b->states[j];
    return OK;
}

ps_status ps_batch_get_stats(const ps_batch *b, ps_batch_stats *out) {
    ps_enter(__func__, __LINE__);
    if (!b || !out) return fail(E_ARG, "null argument");
    *out = b->stats;
    return OK;
}

ps_status ps_batch_destroy(ps_batch *b) {
    ps_enter(__func__, __LINE__);
    if (!b) return OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (ps_circuit *c : b->circs)
        if (c) ps_circuit_destroy(c);
    for (ps_state *h : b->states)
        if (h) ps_destroy(h);
    for (cudaStream_t s : b->branches)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : b->joins)
        if (e) cudaEventDestroy(e);
    for (int r = 0; r < ps_batch::RING; ++r) {
        if (b->h_vals[r]) cudaFreeHost(b->h_vals[r]);
        if (b->copied[r]) cudaEventDestroy(b->copied[r]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->tfork) cudaEventDestroy(b->tfork);
    if (b->tjoin) cudaEventDestroy(b->tjoin);
    if (b->side) cudaStreamDestroy(b->side);
    for (void *p : b->table_mem) cudaFree(p);
    cudaFree(b->d_vals);
    cudaFree(b->d_dst);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return OK;
}

}  // extern "C"

// ================================================================ serving
namespace ps {
namespace {

struct SrvJob {
    uint64_t id = 0;
    std::vector<ps_op> ops;
    std::vector<float> params;
    uint64_t n = 0, shots = 0;
    int64_t seed = 0;
    size_t bytes = 0;
    uint64_t shot_gates = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    uint64_t retry_after = UINT64_MAX;  // re-admit only after this many jobs finished
    bool signs_only = false;            // run on a signs-only state (records are all it returns)
    size_t full_bytes = 0;              // device bytes with per-shot tableaux
    // park / resume: start from a parked tableau (packed words of every
    // shot) and event counter instead of |0...0>; keep the final ones
    bool resume = false, keep = false;
    std::vector<uint64_t> in_x, in_z, in_r, out_x, out_z, out_r;
    uint64_t in_events = 0, out_events = 0;
    bool done = false;
    int status = OK;
    std::string err;
    uint64_t nm = 0, words = 0;
    std::vector<uint64_t> res, det;
    uint64_t *pin_res = nullptr, *pin_det = nullptr;  // records in the server's pinned pool (else res / det)
    size_t rec_words = 0;
};

}  // namespace
}  // namespace ps

struct ps_server {
    ps_server_options opts{};
    int device = 0;
    ps::DevPool pool;
    void *region = nullptr;
    // Pinned host memory for finished jobs' records: the device-to-host copy
    // runs at DMA speed into pages that are resident already.
    ps::DevPool hpool;
    void *hregion = nullptr;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ps::SrvJob *> queue;
    std::unordered_map<uint64_t, std::unique_ptr<ps::SrvJob>> jobs;
    size_t reserved = 0;
    int active = 0;
    bool stop = false;
    uint64_t next_id = 1, submitted = 0, completed = 0, failed = 0, cancelled = 0, shot_gates = 0;
    uint64_t tableau_jobs = 0;
    uint64_t finished = 0;  // completed + failed: the jobs that gave their memory back
    std::vector<double> latencies;
    double first_submit = -1.0, last_done = 0.0;
    std::vector<std::thread> workers;
};

namespace ps {
namespace {

// First queued job that fits the budget and a free slot, in arrival order;
// a head job that has waited longer than hol_wait_s is not overtaken.
SrvJob *pick_job(ps_server *s, double now) {
    if (s->active >= s->opts.max_active) return nullptr;
    for (size_t i = 0; i < s->queue.size(); ++i) {
        SrvJob *j = s->queue[i];
        const bool waiting_retry = j->retry_after != UINT64_MAX && s->finished <= j->retry_after;
        if (!waiting_retry && s->reserved + j->bytes <= s->pool.cap) {
            s->queue.erase(s->queue.begin() + (std::ptrdiff_t)i);
            return j;
        }
        if (i == 0 && s->opts.hol_wait_s >= 0 && now - j->t_submit > s->opts.hol_wait_s) return nullptr;
    }
    return nullptr;
}

// run_job: the circuit needs per-shot tableaux after all; admit the job
// again with them.
constexpr int kNeedTableau = 1 << 20;

// Runs one admitted job on the calling worker thread: state from the pool,
// fused compile, one run from |0...0>, records to host, everything returned.
int run_job(ps_server *s, SrvJob *j) {
    NvtxRange range("ps served job " + std::to_string(j->id));
    ps_state *h = new ps_state;
    ps_circuit *c = nullptr;
    int rc = state_alloc(h, (int64_t)j->n, (int64_t)j->shots, j->seed, &s->pool, j->signs_only);
    if (rc == OK && j->resume) {  // the parked tableau and event counter
        const size_t plane = j->in_x.size() * sizeof(uint64_t), rb = j->in_r.size() * sizeof(uint64_t);
        cudaError_t e = cudaMemcpyAsync(h->X, j->in_x.data(), plane, cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h->Z, j->in_z.data(), plane, cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h->R, j->in_r.data(), rb, cudaMemcpyHostToDevice, h->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "resume copy");
        h->events = j->in_events;
    }
    if (rc == OK) {
        h->valid = !j->resume;
        ps_circuit_options co{};
        co.mode = PS_MODE_FUSED;
        co.use_graph = 0;
        rc = ps_circuit_compile(h, j->ops.data(), j->ops.size(), j->params.data(), j->params.size(), &co, &c);
        if (rc == E_STATE && j->signs_only) rc = kNeedTableau;
    }
    if (rc == OK && s->opts.autotune) rc = ps_circuit_autotune(c, nullptr, nullptr);
    if (rc == OK) rc = ps_circuit_run(c, j->resume ? 0 : 1);
    if (rc == OK) {
        ps_circuit_stats cs{};
        ps_circuit_get_stats(c, &cs);
        j->nm = cs.num_measurements;
        j->words = (uint64_t)h->w;
        j->rec_words = j->nm * j->words;
        const size_t rb = j->rec_words * sizeof(uint64_t);
        void *pr = nullptr, *pd = nullptr;
        if (rb && s->hpool.cap && s->hpool.alloc(&pr, rb) && !s->hpool.alloc(&pd, rb)) {
            s->hpool.release(pr);
            pr = nullptr;
        }
        uint64_t wds = 0;
        if (pr) {
            j->pin_res = static_cast<uint64_t *>(pr);
            j->pin_det = static_cast<uint64_t *>(pd);
            rc = ps_circuit_copy_records(c, j->pin_res, j->pin_det, &wds);
        } else {
            // (filled first: with the buffers left unfilled, the copy into pages
            // never touched before made the serving capacity fall by a third)
            j->res.assign(j->rec_words, 0);
            j->det.assign(j->rec_words, 0);
            rc = ps_circuit_copy_records(c, j->res.data(), j->det.data(), &wds);
        }
        if (rc != OK && j->pin_res) {  // a failed job keeps no records
            s->hpool.release(j->pin_res);
            s->hpool.release(j->pin_det);
            j->pin_res = j->pin_det = nullptr;
        }
    }
    if (rc == OK && j->keep) {  // park: the final tableau and event counter to host memory
        const size_t plane = (size_t)h->W * (size_t)h->n * (size_t)h->w, rw = (size_t)h->W * (size_t)h->w;
        j->out_x.resize(plane);
        j->out_z.resize(plane);
        j->out_r.resize(rw);
        cudaError_t e = cudaMemcpyAsync(j->out_x.data(), h->X, plane * 8, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(j->out_z.data(), h->Z, plane * 8, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(j->out_r.data(), h->R, rw * 8, cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "park copy");
        j->out_events = h->events;
    }
    if (rc != OK) j->err = ps_last_error();
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (c) ps_circuit_destroy(c);
    state_free(h);
    delete h;
    return rc;
}

void worker_main(ps_server *s) {
    cudaSetDevice(s->device);
    for (;;) {
        SrvJob *j = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || (j = pick_job(s, seconds_since(s->t0))) != nullptr; });
            if (!j) return;  // stopping
            s->reserved += j->bytes;
            s->active++;
            j->t_admit = seconds_since(s->t0);
        }
        const int rc = run_job(s, j);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->reserved -= j->bytes;
            s->active--;
            if (rc == kNeedTableau && j->full_bytes <= s->pool.cap) {
                j->signs_only = false;
                j->bytes = j->full_bytes;
                j->err.clear();
                s->queue.push_front(j);
            } else if (rc == kNeedTableau) {
                j->status = E_NOMEM;
                j->err = "job needs " + std::to_string(j->full_bytes >> 20) +
                         " MiB of per-shot tableaux, more than the whole HBM budget";
                j->t_done = seconds_since(s->t0);
                j->done = true;
                s->finished++;
                s->failed++;
            } else if (rc == E_NOMEM && s->active > 0) {
                // The pool is fragmented right now: wait for another job to finish.
                j->retry_after = s->finished;
                j->err.clear();
                s->queue.push_front(j);
            } else {
                j->status = rc;
                j->t_done = seconds_since(s->t0);
                j->done = true;
                std::vector<uint64_t>().swap(j->in_x);  // the parked input is no longer needed
                std::vector<uint64_t>().swap(j->in_z);
                std::vector<uint64_t>().swap(j->in_r);
                s->finished++;
                if (rc == OK) {
                    s->completed++;
                    if (!j->signs_only) s->tableau_jobs++;
                    s->shot_gates += j->shot_gates;
                    s->latencies.push_back(j->t_done - j->t_submit);
                    s->last_done = std::max(s->last_done, j->t_done);
                } else {
                    s->failed++;  // its latency is not counted
                }
            }
        }
        s->cv_work.notify_all();
        s->cv_done.notify_all();
    }
}

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = q * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace
}  // namespace ps

extern "C" {

ps_status ps_server_create(const ps_server_options *opts, ps_server **out) {
    ps_enter(__func__, __LINE__);
    if (!opts || !out) return fail(E_ARG, "null argument");
    *out = nullptr;
    if (opts->hbm_budget_bytes < (1u << 20)) return fail(E_ARG, "HBM budget below 1 MiB");
    auto *s = new ps_server;
    s->opts = *opts;
    if (s->opts.max_active <= 0) s->opts.max_active = 16;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e == cudaSuccess) e = cudaMalloc(&s->region, opts->hbm_budget_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return fail(E_NOMEM, std::string("cannot reserve the HBM budget: ") + cudaGetErrorString(e));
    }
    s->pool.reset(s->region, opts->hbm_budget_bytes);
    {  // the pinned record pool (without it, records go to pageable memory)
        const size_t hb = opts->host_pool_bytes ? (size_t)opts->host_pool_bytes : (size_t)1 << 30;
        if (cudaMallocHost(&s->hregion, hb) == cudaSuccess) {
            s->hpool.reset(s->hregion, hb);
        } else {
            cudaGetLastError();
            s->hregion = nullptr;
        }
    }
    s->t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < s->opts.max_active; ++i) s->workers.emplace_back(worker_main, s);
    *out = s;
    return OK;
}

ps_status ps_server_submit(ps_server *s, const ps_job_desc *job, uint64_t *job_id) {
    return ps_server_submit_parked(s, job, nullptr, job_id);
}

ps_status ps_server_submit_parked(ps_server *s, const ps_job_desc *job, const ps_job_park *park, uint64_t *job_id) {
    ps_enter(__func__, __LINE__);
    if (!s || !job) return fail(E_ARG, "null argument");
    TRY(check_job(*job, 0));
    if (park && ((park->x != nullptr) != (park->z != nullptr) || (park->x != nullptr) != (park->r != nullptr)))
        return fail(E_ARG, "a parked tableau needs x, z and r");
    auto j = std::make_unique<SrvJob>();
    if (park) {
        j->keep = park->keep_tableau != 0;
        if (park->x) {
            int64_t w = ((int64_t)job->shots + 63) / 64;
            w = (w + 1) & ~int64_t(1);
            const size_t W = 2 * (size_t)job->num_qubits + 1, plane = W * (size_t)job->num_qubits * (size_t)w;
            j->resume = true;
            j->in_x.assign(park->x, park->x + plane);
            j->in_z.assign(park->z, park->z + plane);
            j->in_r.assign(park->r, park->r + W * (size_t)w);
            j->in_events = park->events;
        }
    }
    j->ops.assign(job->ops, job->ops + job->nops);
    if (job->params && job->nparams) j->params.assign(job->params, job->params + job->nparams);
    j->n = job->num_qubits;
    j->shots = job->shots;
    j->seed = job->seed;
    j->signs_only = !j->resume && !j->keep && signs_only_job(*job);
    j->full_bytes = job_device_bytes(*job, false);
    j->bytes = job_device_bytes(*job, j->signs_only);
    j->shot_gates = count_gates(job->ops, job->nops) * job->shots;
    if (j->bytes > s->pool.cap)
        return fail(E_NOMEM, "job needs " + std::to_string(j->bytes >> 20) + " MiB, more than the whole HBM budget");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return fail(E_STATE, "server is shutting down");
        j->id = s->next_id++;
        j->t_submit = seconds_since(s->t0);
        if (s->first_submit < 0) s->first_submit = j->t_submit;
        s->submitted++;
        if (job_id) *job_id = j->id;
        s->queue.push_back(j.get());
        s->jobs.emplace(j->id, std::move(j));
    }
    s->cv_work.notify_one();
    return OK;
}

ps_status ps_server_wait(ps_server *s, uint64_t job_id, double timeout_s, ps_job_result *out) {
    ps_enter(__func__, __LINE__);
    if (!s) return fail(E_ARG, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return fail(E_RANGE, "unknown job id");
    SrvJob *j = it->second.get();
    auto ready = [&] { return j->done; };
    if (timeout_s < 0)
        s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
        return fail(E_TIMEOUT, "job not finished within the timeout");
    if (out) {
        std::memset(out, 0, sizeof(*out));
        out->status = j->status;
        out->num_measurements = j->nm;
        out->words = j->words;
        out->shot_gates = j->shot_gates;
        out->device_bytes = j->bytes;
        out->submit_s = j->t_submit;
        out->admit_s = j->t_admit;
        out->done_s = j->t_done;
        out->latency_s = j->t_done - j->t_submit;
    }
    if (j->status != OK) return fail(j->status, "job " + std::to_string(job_id) + " failed: " + j->err);
    return OK;
}

ps_status ps_server_copy_records(ps_server *s, uint64_t job_id, uint64_t *results, uint64_t *determined) {
    ps_enter(__func__, __LINE__);
    if (!s) return fail(E_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return fail(E_RANGE, "unknown job id");
    SrvJob *j = it->second.get();
    if (!j->done) return fail(E_STATE, "job not finished");
    if (j->status != OK) return fail(j->status, "job failed: " + j->err);
    const uint64_t *rs = j->pin_res ? j->pin_res : j->res.data(), *ds = j->pin_res ? j->pin_det : j->det.data();
    if (results && j->rec_words) std::memcpy(results, rs, j->rec_words * sizeof(uint64_t));
    if (determined && j->rec_words) std::memcpy(determined, ds, j->rec_words * sizeof(uint64_t));
    return OK;
}

ps_status ps_server_copy_tableau(ps_server *s, uint64_t job_id, uint64_t *x, uint64_t *z, uint64_t *r,
                                 uint64_t *events) {
    ps_enter(__func__, __LINE__);
    if (!s) return fail(E_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return fail(E_RANGE, "unknown job id");
    SrvJob *j = it->second.get();
    if (!j->done) return fail(E_STATE, "job not finished");
    if (j->status != OK) return fail(j->status, "job failed: " + j->err);
    if (!j->keep) return fail(E_STATE, "the job was not submitted to keep its tableau");
    if (x) std::memcpy(x, j->out_x.data(), j->out_x.size() * sizeof(uint64_t));
    if (z) std::memcpy(z, j->out_z.data(), j->out_z.size() * sizeof(uint64_t));
    if (r) std::memcpy(r, j->out_r.data(), j->out_r.size() * sizeof(uint64_t));
    if (events) *events = j->out_events;
    return OK;
}

ps_status ps_server_release(ps_server *s, uint64_t job_id) {
    ps_enter(__func__, __LINE__);
    if (!s) return fail(E_ARG, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return fail(E_RANGE, "unknown job id");
    if (!it->second->done) return fail(E_STATE, "job not finished");
    if (it->second->pin_res) {
        s->hpool.release(it->second->pin_res);
        s->hpool.release(it->second->pin_det);
    }
    s->jobs.erase(it);
    return OK;
}

ps_status ps_server_cancel(ps_server *s, uint64_t job_id) {
    ps_enter(__func__, __LINE__);
    if (!s) return fail(E_ARG, "null server");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) return fail(E_RANGE, "unknown job " + std::to_string(job_id));
        SrvJob *j = it->second.get();
        auto q = std::find(s->queue.begin(), s->queue.end(), j);
        if (q == s->queue.end())
            return fail(E_STATE, "job " + std::to_string(job_id) + " is not queued (already admitted or done)");
        s->queue.erase(q);
        j->status = E_STATE;
        j->err = "cancelled before it was admitted";
        j->t_done = seconds_since(s->t0);
        j->done = true;
        s->cancelled++;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    return OK;
}

ps_status ps_server_drain(ps_server *s, double timeout_s) {
    ps_enter(__func__, __LINE__);
    if (!s) return fail(E_ARG, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto idle = [&] { return s->queue.empty() && s->active == 0; };
    if (timeout_s < 0)
        s->cv_done.wait(lk, idle);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), idle))
        return fail(E_TIMEOUT, "jobs still queued or active");
    return OK;
}

ps_status ps_server_get_stats(ps_server *s, ps_server_stats *out) {
    ps_enter(__func__, __LINE__);
    if (!s || !out) return fail(E_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->cancelled = s->cancelled;
    out->tableau_jobs = s->tableau_jobs;
    out->queued = s->queue.size();
    out->active = (uint64_t)s->active;
    out->shot_gates_completed = s->shot_gates;
    {
        std::lock_guard<std::mutex> pk(s->pool.mu);
        out->pool_bytes = s->pool.cap;
        out->pool_peak_bytes = s->pool.peak;
    }
    out->p50_latency_s = percentile(s->latencies, 0.50);
    out->p99_latency_s = percentile(s->latencies, 0.99);
    if (!s->latencies.empty()) {
        out->mean_latency_s = std::accumulate(s->latencies.begin(), s->latencies.end(), 0.0) / s->latencies.size();
        out->max_latency_s = *std::max_element(s->latencies.begin(), s->latencies.end());
    }
    out->first_submit_s = s->first_submit;
    out->last_done_s = s->last_done;
    return OK;
}

ps_status ps_server_now(const ps_server *s, double *seconds) {
    ps_enter(__func__, __LINE__);
    if (!s || !seconds) return fail(E_ARG, "null argument");
    *seconds = seconds_since(s->t0);
    return OK;
}

ps_status ps_server_destroy(ps_server *s) {
    ps_enter(__func__, __LINE__);
    if (!s) return OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (SrvJob *j : s->queue) {  // never admitted
            j->done = true;
            j->status = E_STATE;
            j->err = "server destroyed before the job was admitted";
        }
        s->queue.clear();
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    s->cv_done.notify_all();
    cudaFree(s->region);
    if (s->hregion) cudaFreeHost(s->hregion);
    delete s;
    return OK;
}

}  // extern "C"
