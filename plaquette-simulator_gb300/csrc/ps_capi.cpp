// ps_capi.cpp -- the extern "C" boundary (include/plaquette_gpu.h): argument
// checks, record bookkeeping and error reporting around the CUDA launches.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/plaquette_gpu.h"
#include "ps_internal.h"

namespace ps {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

// Error.hpp:91-98 message format: "[file][Line:N][Method:f]: Error in
// Plaquette: msg".  The location is the C-ABI entry point that failed.
static thread_local const char *g_method = "";
static thread_local int g_line = 0;

int fail(int status, const std::string &msg) {
    g_last_error = std::string("[plaquette_gpu][Line:") + std::to_string(g_line) + "][Method:" + g_method +
                   "]: Error in Plaquette: " + msg;
    return status;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void ps_enter(const char *method, int line) {
    g_method = method;
    g_line = line;
    g_last_error.clear();
}

}  // namespace ps

using namespace ps;

#define ENTER()                 \
    ps::g_method = __func__;    \
    ps::g_line = __LINE__;      \
    ps::g_last_error.clear()

#define CHECK_HANDLE(h) \
    if (!(h)) return fail(E_ARG, "null handle")

#define CHECK_QUBIT(h, q) \
    if ((int64_t)(q) < 0 || (int64_t)(q) >= (h)->n) return fail(E_ARG, "qubit " + std::to_string(q) + " out of range")

#define TRY(expr)                     \
    do {                              \
        int _rc = (expr);             \
        if (_rc != OK) return _rc;    \
    } while (0)

namespace {

// Work still queued when the process exits must finish before the CUDA
// runtime unregisters this library's kernels; the handler is registered
// after the runtime initialised, so it runs before the runtime's own.
void drain_at_exit() { cudaDeviceSynchronize(); }

ps_status create_common(uint64_t n, uint64_t S, int64_t seed, ps_state **out) {
    static std::once_flag exit_hook;
    std::call_once(exit_hook, [] {
        cudaFree(nullptr);  // initialise the runtime first
        std::atexit(drain_at_exit);
    });
    if (!out) return fail(E_ARG, "null output pointer");
    *out = nullptr;
    if (n > (uint64_t)1 << 20 || S > (uint64_t)1 << 36) return fail(E_ARG, "num_qubits or batch_size too large");
    auto *h = new ps_state;
    int rc = state_alloc(h, (int64_t)n, (int64_t)S, seed);
    if (rc != OK) {
        state_free(h);
        delete h;
        return rc;
    }
    *out = h;
    return OK;
}

int measure_one(ps_state *h, int64_t q, float bias, int64_t id, const uint8_t *forced, int reset, uint64_t *out_id) {
    int64_t rid = id;
    if (id < 0) {
        TRY(record_new(h, q, &rid));
    } else if ((uint64_t)id >= h->recs.size()) {
        return fail(E_RANGE, "Measurement id is out of range.");
    }
    Record &rec = h->recs[(size_t)rid];
    rec.host_valid = false;  // re-measuring into an id replaces its contents
    rec.qubit = q;
    const u64 *dforced = nullptr;
    TRY(upload_forced(h, forced, &dforced));
    MeasOp op{};
    op.q = (int32_t)q;
    op.reset = reset;
    op.bias = bias;
    op.event = (uint32_t)h->events++;
    op.forced = dforced;
    op.res = rec.res;
    op.det = rec.det;
    if (h->n > 0 && h->S > 0) TRY(launch_measure(h, &op, 1));
    if (out_id) *out_id = (uint64_t)rid;
    return OK;
}

}  // namespace

extern "C" {

const char *ps_last_error(void) { return ps::g_last_error.c_str(); }

const char *ps_version(void) { return "plaquette-gb300 0.1.0"; }

ps_status ps_set_device(int device) {
    ENTER();
    PS_CUDA(cudaSetDevice(device));
    return OK;
}

ps_status ps_device_synchronize(void) {
    ENTER();
    PS_CUDA(cudaDeviceSynchronize());
    return OK;
}

const char *ps_backend_name(void) {
    static std::string name;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDeviceProp prop;
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess)
            name = std::string("CUDA sm_") + std::to_string(prop.major) + std::to_string(prop.minor) + "a (" +
                   prop.name + ")";
        else
            name = "CUDA sm_103a (no device)";
    });
    return name.c_str();
}

ps_status ps_create(uint64_t n, uint64_t S, int64_t seed, int init_zero, ps_state **out) {
    ENTER();
    TRY(create_common(n, S, seed, out));
    if (init_zero && n > 0 && S > 0) {
        int rc = launch_init_zero(*out);
        (*out)->valid = true;
        if (rc != OK) {
            state_free(*out);
            delete *out;
            *out = nullptr;
            return rc;
        }
    } else {
        // Like an uninitialised Kokkos View (zero-filled by Kokkos), the
        // tableau starts all-zero.
        cudaMemsetAsync((*out)->X, 0, (size_t)(*out)->W * (*out)->n * (*out)->w * 8, (*out)->stream);
        cudaMemsetAsync((*out)->Z, 0, (size_t)(*out)->W * (*out)->n * (*out)->w * 8, (*out)->stream);
        cudaMemsetAsync((*out)->R, 0, (size_t)(*out)->W * (*out)->w * 8, (*out)->stream);
    }
    return OK;
}

ps_status ps_create_from_host(const int32_t *x, const int32_t *z, const int32_t *r, uint64_t n, uint64_t S,
                              int64_t seed, ps_state **out) {
    ENTER();
    if (!x || !z || !r) return fail(E_ARG, "null host tableau");
    TRY(create_common(n, S, seed, out));
    int rc = pack_from_host(*out, x, z, r);
    if (rc != OK) {
        state_free(*out);
        delete *out;
        *out = nullptr;
    }
    return rc;
}

ps_status ps_clone(const ps_state *o, ps_state **out) {
    ENTER();
    CHECK_HANDLE(o);
    TRY(create_common((uint64_t)o->n, (uint64_t)o->S, o->seed, out));
    ps_state *h = *out;
    h->events = o->events;
    h->valid = o->valid;
    h->word_base = o->word_base;
    const size_t plane = (size_t)o->W * o->n * o->w * 8;
    PS_CUDA(cudaStreamSynchronize(o->stream));
    PS_CUDA(cudaMemcpyAsync(h->X, o->X, plane, cudaMemcpyDeviceToDevice, h->stream));
    PS_CUDA(cudaMemcpyAsync(h->Z, o->Z, plane, cudaMemcpyDeviceToDevice, h->stream));
    PS_CUDA(cudaMemcpyAsync(h->R, o->R, (size_t)o->W * o->w * 8, cudaMemcpyDeviceToDevice, h->stream));
    return OK;
}

ps_status ps_destroy(ps_state *h) {
    ENTER();
    if (!h) return OK;
    state_free(h);
    delete h;
    return OK;
}

ps_status ps_get_num_qubits(const ps_state *h, uint64_t *out) {
    ENTER();
    CHECK_HANDLE(h);
    *out = (uint64_t)h->n;
    return OK;
}

ps_status ps_get_batch_size(const ps_state *h, uint64_t *out) {
    ENTER();
    CHECK_HANDLE(h);
    *out = (uint64_t)h->S;
    return OK;
}

ps_status ps_get_seed(const ps_state *h, int64_t *out) {
    ENTER();
    CHECK_HANDLE(h);
    *out = h->seed;
    return OK;
}

ps_status ps_get_event_counter(const ps_state *h, uint64_t *out) {
    ENTER();
    CHECK_HANDLE(h);
    *out = h->events;
    return OK;
}

ps_status ps_set_event_counter(ps_state *h, uint64_t events) {
    ENTER();
    CHECK_HANDLE(h);
    h->events = events;
    return OK;
}

ps_status ps_set_shot_offset(ps_state *h, uint64_t first_shot) {
    ENTER();
    CHECK_HANDLE(h);
    if (first_shot % 64) return fail(E_ARG, "shot offset must be a multiple of 64");
    h->word_base = (int64_t)(first_shot / 64);
    return OK;
}

ps_status ps_get_shot_offset(const ps_state *h, uint64_t *first_shot) {
    ENTER();
    CHECK_HANDLE(h);
    if (!first_shot) return fail(E_ARG, "null output pointer");
    *first_shot = (uint64_t)h->word_base * 64;
    return OK;
}

ps_status ps_reset(ps_state *h) {
    ENTER();
    CHECK_HANDLE(h);
    h->valid = true;
    if (h->n == 0 || h->S == 0) return OK;
    return launch_init_zero(h);
}

ps_status ps_checksum(ps_state *h, int64_t s0, int64_t s1, int64_t *out) {
    ENTER();
    CHECK_HANDLE(h);
    if (!out) return fail(E_ARG, "null output pointer");
    if (s1 < 0) s1 = h->S;
    if (s0 < 0 || s0 > s1 || s1 > h->S) return fail(E_ARG, "shot range out of bounds");
    return checksum(h, s0, s1, out);
}

ps_status ps_device_to_host(ps_state *h, int32_t *x, int32_t *z, int32_t *r) {
    ENTER();
    CHECK_HANDLE(h);
    if (!x || !z || !r) return fail(E_ARG, "null host buffer");
    return unpack_to_host(h, x, z, r);
}

ps_status ps_host_to_device(ps_state *h, const int32_t *x, const int32_t *z, const int32_t *r) {
    ENTER();
    CHECK_HANDLE(h);
    if (!x || !z || !r) return fail(E_ARG, "null host buffer");
    h->valid = false;
    return pack_from_host(h, x, z, r);
}

#define GATE1(NAME, CODE)                          \
    ps_status NAME(ps_state *h, uint64_t q) {      \
        ENTER();                                   \
        CHECK_HANDLE(h);                           \
        CHECK_QUBIT(h, q);                         \
        return launch_gate(h, CODE, (int64_t)q, 0, nullptr); \
    }
GATE1(ps_h, OP_H)
GATE1(ps_s, OP_S)
GATE1(ps_x, OP_X)
GATE1(ps_y, OP_Y)
GATE1(ps_z, OP_Z)
#undef GATE1

ps_status ps_cx(ps_state *h, uint64_t c, uint64_t t) {
    ENTER();
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, c);
    CHECK_QUBIT(h, t);
    if (c == t) return fail(E_ARG, "control and target must differ");
    return launch_gate(h, OP_CX, (int64_t)c, (int64_t)t, nullptr);
}

ps_status ps_cz(ps_state *h, uint64_t c, uint64_t t) {
    ENTER();
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, c);
    CHECK_QUBIT(h, t);
    if (c == t) return fail(E_ARG, "control and target must differ");
    return launch_gate(h, OP_CZ, (int64_t)c, (int64_t)t, nullptr);
}

ps_status ps_apply_to_qubits(ps_state *h, int32_t code, const uint64_t *targets, uint64_t count) {
    ENTER();
    CHECK_HANDLE(h);
    if (count && !targets) return fail(E_ARG, "null targets");
    const bool two = code == OP_CX || code == OP_CZ;
    if (!(code >= OP_H && code <= OP_CZ)) return fail(E_ARG, "op code is not a gate");
    if (two && (count % 2)) return fail(E_ARG, "two-qubit gates need an even number of targets");
    for (uint64_t k = 0; k < count; ++k) CHECK_QUBIT(h, targets[k]);
    for (uint64_t k = 0; k < count; k += two ? 2 : 1) {
        if (two && targets[k] == targets[k + 1]) return fail(E_ARG, "control and target must differ");
        TRY(launch_gate(h, code, (int64_t)targets[k], two ? (int64_t)targets[k + 1] : 0, nullptr));
    }
    return OK;
}

ps_status ps_h_flag(ps_state *h, uint64_t q, uint64_t id) {
    ENTER();
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, q);
    if (id >= h->recs.size()) return fail(E_RANGE, "Measurement id is out of range.");
    return launch_gate(h, OP_H_IF, (int64_t)q, 0, h->recs[(size_t)id].res);
}

ps_status ps_s_flag(ps_state *h, uint64_t q, uint64_t id) {
    ENTER();
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, q);
    if (id >= h->recs.size()) return fail(E_RANGE, "Measurement id is out of range.");
    return launch_gate(h, OP_S_IF, (int64_t)q, 0, h->recs[(size_t)id].res);
}

ps_status ps_measure(ps_state *h, uint64_t q, float bias, int64_t id, const uint8_t *forced, uint64_t *out_id) {
    ENTER();
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, q);
    return measure_one(h, (int64_t)q, bias, id, forced, 0, out_id);
}

ps_status ps_measure_qubits(ps_state *h, const uint64_t *targets, uint64_t count, float bias, uint64_t *first_id) {
    ENTER();
    CHECK_HANDLE(h);
    if (count && !targets) return fail(E_ARG, "null targets");
    for (uint64_t k = 0; k < count; ++k) CHECK_QUBIT(h, targets[k]);
    if (first_id) *first_id = (uint64_t)h->recs.size();
    for (uint64_t k = 0; k < count; ++k) TRY(measure_one(h, (int64_t)targets[k], bias, -1, nullptr, 0, nullptr));
    return OK;
}

ps_status ps_reset_qubit(ps_state *h, uint64_t q, const uint8_t *forced, uint64_t *out_id) {
    ENTER();
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, q);
    return measure_one(h, (int64_t)q, 0.5f, -1, forced, 1, out_id);
}

ps_status ps_get_measurement(ps_state *h, uint64_t id, uint64_t shot, int32_t *res, int32_t *det) {
    ENTER();
    CHECK_HANDLE(h);
    if (id >= h->recs.size() || shot >= (uint64_t)h->S)
        return fail(E_RANGE, "Measurement id or batch index is out of range.");
    TRY(record_fetch(h, (int64_t)id));
    const Record &rec = h->recs[(size_t)id];
    if (res) *res = (int32_t)((rec.host_res[shot >> 6] >> (shot & 63)) & 1ull);
    if (det) *det = (int32_t)((rec.host_det[shot >> 6] >> (shot & 63)) & 1ull);
    return OK;
}

ps_status ps_get_record_bits(ps_state *h, uint64_t id, uint8_t *res_bits, uint8_t *det_bits) {
    ENTER();
    CHECK_HANDLE(h);
    if (id >= h->recs.size()) return fail(E_RANGE, "Measurement id is out of range.");
    TRY(record_fetch(h, (int64_t)id));
    const Record &rec = h->recs[(size_t)id];
    const size_t nb = (size_t)(h->S + 7) / 8;
    if (res_bits) std::memcpy(res_bits, rec.host_res.data(), nb);
    if (det_bits) std::memcpy(det_bits, rec.host_det.data(), nb);
    if (h->S % 8) {
        const uint8_t keep = (uint8_t)((1u << (h->S % 8)) - 1u);
        if (res_bits) res_bits[nb - 1] &= keep;
        if (det_bits) det_bits[nb - 1] &= keep;
    }
    return OK;
}

ps_status ps_num_records(const ps_state *h, uint64_t *out) {
    ENTER();
    CHECK_HANDLE(h);
    *out = (uint64_t)h->recs.size();
    return OK;
}

ps_status ps_record_qubit(const ps_state *h, uint64_t id, uint64_t *out) {
    ENTER();
    CHECK_HANDLE(h);
    if (id >= h->recs.size()) return fail(E_RANGE, "Measurement id is out of range.");
    *out = (uint64_t)h->recs[(size_t)id].qubit;
    return OK;
}

ps_status ps_pauli_channel_1(ps_state *h, uint64_t q, const float p[3]) {
    ENTER();
    if (!p) return fail(E_ARG, "null probabilities");
    TRY(check_channel_probs(p, 3));
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, q);
    uint64_t thr[4];
    channel_thresholds(p, 3, thr);
    return launch_pauli_channel(h, (int64_t)q, 0, thr, 3);
}

ps_status ps_pauli_channel_1_noalloc(ps_state *h, uint64_t q, const float p[3]) {
    ENTER();
    if (!p) return fail(E_ARG, "null probabilities");
    TRY(check_channel_probs(p, 3));
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, q);
    uint64_t thr[4];
    channel_thresholds(p, 3, thr);
    return launch_pauli_channel_noalloc(h, (int64_t)q, thr);
}

ps_status ps_pauli_channel_2(ps_state *h, uint64_t a, uint64_t b, const float p[15]) {
    ENTER();
    if (!p) return fail(E_ARG, "null probabilities");
    TRY(check_channel_probs(p, 15));
    CHECK_HANDLE(h);
    CHECK_QUBIT(h, a);
    CHECK_QUBIT(h, b);
    if (a == b) return fail(E_ARG, "two-qubit channel needs distinct qubits");
    uint64_t thr[16];
    channel_thresholds(p, 15, thr);
    return launch_pauli_channel(h, (int64_t)a, (int64_t)b, thr, 15);
}

ps_status ps_synchronize(ps_state *h) {
    ENTER();
    CHECK_HANDLE(h);
    PS_CUDA(cudaStreamSynchronize(h->stream));
    return OK;
}

ps_status ps_get_stream(const ps_state *h, void **stream) {
    ENTER();
    CHECK_HANDLE(h);
    *stream = (void *)h->stream;
    return OK;
}

ps_status ps_get_device_tableau(const ps_state *h, void **x, void **z, void **r, uint64_t *words) {
    ENTER();
    CHECK_HANDLE(h);
    if (x) *x = h->X;
    if (z) *z = h->Z;
    if (r) *r = h->R;
    if (words) *words = (uint64_t)h->w;
    return OK;
}

ps_status ps_copy_tableau_words(ps_state *h, uint64_t first_word, uint64_t nwords, uint64_t *x, uint64_t *z,
                                uint64_t *r) {
    ENTER();
    CHECK_HANDLE(h);
    if (nwords > (uint64_t)h->w || first_word > (uint64_t)h->w - nwords)
        return fail(E_RANGE, "word range outside the state");
    if (nwords == 0 || h->n == 0) return OK;
    if (h->signs_only && (x || z)) return fail(E_STATE, "a signs-only state holds no x / z");
    const size_t width = nwords * sizeof(u64), spitch = (size_t)h->w * sizeof(u64);
    const size_t rows = (size_t)h->W * (size_t)h->n;
    if (x) PS_CUDA(cudaMemcpy2DAsync(x, width, h->X + first_word, spitch, width, rows, cudaMemcpyDeviceToHost, h->stream));
    if (z) PS_CUDA(cudaMemcpy2DAsync(z, width, h->Z + first_word, spitch, width, rows, cudaMemcpyDeviceToHost, h->stream));
    if (r)
        PS_CUDA(cudaMemcpy2DAsync(r, width, h->R + first_word, spitch, width, (size_t)h->W, cudaMemcpyDeviceToHost,
                                  h->stream));
    PS_CUDA(cudaStreamSynchronize(h->stream));
    return OK;
}

ps_status ps_load_tableau_words(ps_state *h, uint64_t first_word, uint64_t nwords, const uint64_t *x,
                                const uint64_t *z, const uint64_t *r) {
    ENTER();
    CHECK_HANDLE(h);
    if (nwords > (uint64_t)h->w || first_word > (uint64_t)h->w - nwords)
        return fail(E_RANGE, "word range outside the state");
    if (h->signs_only) return fail(E_STATE, "a signs-only state holds no x / z");
    if (nwords == 0 || h->n == 0) return OK;
    h->valid = false;  // not known to come from |0...0> through gates and measurements
    const size_t width = nwords * sizeof(u64), dpitch = (size_t)h->w * sizeof(u64);
    const size_t rows = (size_t)h->W * (size_t)h->n;
    if (x) PS_CUDA(cudaMemcpy2DAsync(h->X + first_word, dpitch, x, width, width, rows, cudaMemcpyHostToDevice, h->stream));
    if (z) PS_CUDA(cudaMemcpy2DAsync(h->Z + first_word, dpitch, z, width, width, rows, cudaMemcpyHostToDevice, h->stream));
    if (r)
        PS_CUDA(cudaMemcpy2DAsync(h->R + first_word, dpitch, r, width, width, (size_t)h->W, cudaMemcpyHostToDevice,
                                  h->stream));
    PS_CUDA(cudaStreamSynchronize(h->stream));  // the host buffers may go once this returns
    return OK;
}

ps_status ps_device_to_device(ps_state *h, const void *x, const void *z, const void *r) {
    ENTER();
    CHECK_HANDLE(h);
    if (!x || !z || !r) return fail(E_ARG, "null device plane");
    if (h->signs_only) return fail(E_STATE, "a signs-only state holds no x / z");
    h->valid = false;
    const size_t plane = (size_t)h->W * (size_t)(h->n > 0 ? h->n : 1) * (size_t)h->w * sizeof(u64);
    PS_CUDA(cudaMemcpyAsync(h->X, x, plane, cudaMemcpyDeviceToDevice, h->stream));
    PS_CUDA(cudaMemcpyAsync(h->Z, z, plane, cudaMemcpyDeviceToDevice, h->stream));
    PS_CUDA(cudaMemcpyAsync(h->R, r, (size_t)h->W * (size_t)h->w * sizeof(u64), cudaMemcpyDeviceToDevice, h->stream));
    PS_CUDA(cudaStreamSynchronize(h->stream));
    return OK;
}

ps_status ps_get_record_device(ps_state *h, uint64_t id, void **results, void **determined) {
    ENTER();
    CHECK_HANDLE(h);
    if (id >= h->recs.size()) return fail(E_RANGE, "Measurement id is out of range.");
    if (results) *results = h->recs[(size_t)id].res;
    if (determined) *determined = h->recs[(size_t)id].det;
    return OK;
}

}  // extern "C"
