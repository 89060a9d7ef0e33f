// ref_capi.cpp -- C entry points over the reference's own CliffordState<int>
// (test infrastructure only).
//
// Compiled, by oracle/Makefile, against the reference's headers where they lie
// (plaquette_simulator/src/CliffordState.hpp and the functor headers it
// includes), unmodified, with the project's Kokkos-API shim (kokkos_shim/) on
// the include path.  The result, oracle/_ref/libplaquette_ref.so, is the
// reference itself running on OpenMP; the tests use it to pin the C
// restatement (ps_oracle.c) shot-for-shot under forced random outcomes.
#include <Kokkos_Core.hpp>
#include <Kokkos_Random.hpp>

#include "CliffordState.hpp"
#include "ps_oracle.h"

#include <cstdint>
#include <vector>

using Plaquette::CliffordState;

namespace {
struct RefHandle {
    CliffordState<int> *st;
    std::int64_t seed;
    std::int64_t shot_base;
    std::uint64_t events;
};

// Forced draws are installed for exactly one MeasureQubit call.
struct ForcedScope {
    explicit ForcedScope(const std::uint8_t *bits) { Kokkos::shim::forced_bits() = bits; }
    ~ForcedScope() { Kokkos::shim::forced_bits() = nullptr; }
};

Kokkos::View<int *> flag_view(const std::vector<int> &f) {
    Kokkos::View<int *> v("flag", f.size());
    for (size_t k = 0; k < f.size(); ++k) v(k) = f[k];
    return v;
}

void cond_paulis(RefHandle *h, size_t q, const std::vector<int> &fx, const std::vector<int> &fz) {
    auto vx = flag_view(fx);
    auto vz = flag_view(fz);
    h->st->ApplyHadamardGateWithApplyFlag(q, vx);
    h->st->ApplyPhaseGateWithApplyFlag(q, vx);
    h->st->ApplyPhaseGateWithApplyFlag(q, vx);
    h->st->ApplyHadamardGateWithApplyFlag(q, vx);
    h->st->ApplyPhaseGateWithApplyFlag(q, vz);
    h->st->ApplyPhaseGateWithApplyFlag(q, vz);
}

} // namespace

extern "C" {

void *ref_create(std::int64_t n, std::int64_t batch, std::int64_t seed, int init_zero, std::int64_t shot_base) {
    auto *h = new RefHandle;
    h->st = new CliffordState<int>(static_cast<size_t>(n), static_cast<size_t>(batch), static_cast<int>(seed),
                                   init_zero != 0);
    h->seed = h->st->GetSeed();
    h->shot_base = shot_base;
    h->events = 0;
    return h;
}

void *ref_create_from_host(const std::int32_t *x, const std::int32_t *z, const std::int32_t *r, std::int64_t n,
                           std::int64_t batch, std::int64_t seed) {
    const size_t W = 2 * static_cast<size_t>(n) + 1;
    std::vector<int> xv(x, x + batch * W * n), zv(z, z + batch * W * n), rv(r, r + batch * W);
    auto *h = new RefHandle;
    h->st = new CliffordState<int>(xv, zv, rv, static_cast<size_t>(n), static_cast<size_t>(batch), seed);
    h->seed = h->st->GetSeed();
    h->shot_base = 0;
    h->events = 0;
    return h;
}

void ref_destroy(void *p) {
    auto *h = static_cast<RefHandle *>(p);
    delete h->st;
    delete h;
}

void ref_h(void *p, std::int64_t q) { static_cast<RefHandle *>(p)->st->ApplyHadamardGate(q); }
void ref_s(void *p, std::int64_t q) { static_cast<RefHandle *>(p)->st->ApplyPhaseGate(q); }
void ref_x(void *p, std::int64_t q) { static_cast<RefHandle *>(p)->st->ApplyPauliXGate(q); }
void ref_y(void *p, std::int64_t q) { static_cast<RefHandle *>(p)->st->ApplyPauliYGate(q); }
void ref_z(void *p, std::int64_t q) { static_cast<RefHandle *>(p)->st->ApplyPauliZGate(q); }
void ref_cx(void *p, std::int64_t c, std::int64_t t) { static_cast<RefHandle *>(p)->st->ApplyControlNotGate(c, t); }
void ref_cz(void *p, std::int64_t c, std::int64_t t) { static_cast<RefHandle *>(p)->st->ApplyControlPhaseGate(c, t); }

void ref_h_flag(void *p, std::int64_t q, std::int64_t rec) {
    auto *h = static_cast<RefHandle *>(p);
    h->st->ApplyHadamardGateWithApplyFlag(q, *h->st->GetMeasurement(rec).measurement_results_device);
}
void ref_s_flag(void *p, std::int64_t q, std::int64_t rec) {
    auto *h = static_cast<RefHandle *>(p);
    h->st->ApplyPhaseGateWithApplyFlag(q, *h->st->GetMeasurement(rec).measurement_results_device);
}

std::int64_t ref_measure(void *p, std::int64_t q, float bias, std::int64_t id, const std::uint8_t *forced) {
    auto *h = static_cast<RefHandle *>(p);
    ForcedScope scope(forced);
    h->events++;
    try {
        if (id < 0) return static_cast<std::int64_t>(h->st->MeasureQubit(q, bias));
        return static_cast<std::int64_t>(h->st->MeasureQubit(q, bias, static_cast<size_t>(id)));
    } catch (const Plaquette::Exception &) {
        return -1;
    }
}

std::int64_t ref_reset_qubit(void *p, std::int64_t q, const std::uint8_t *forced) {
    std::int64_t rid = ref_measure(p, q, 0.5f, -1, forced);
    ref_h_flag(p, q, rid);
    ref_s_flag(p, q, rid);
    ref_s_flag(p, q, rid);
    ref_h_flag(p, q, rid);
    return rid;
}

int ref_get_measurement(void *p, std::int64_t id, std::int64_t shot, std::int32_t *res, std::int32_t *det) {
    auto v = static_cast<RefHandle *>(p)->st->GetMeasurement(static_cast<size_t>(id), static_cast<size_t>(shot));
    if (!v.has_value()) return -1;
    *res = v->first;
    *det = v->second;
    return 0;
}

void ref_device_to_host(void *p, std::int32_t *x, std::int32_t *z, std::int32_t *r) {
    auto &&[xv, zv, rv] = static_cast<RefHandle *>(p)->st->DeviceToHost();
    std::copy(xv.begin(), xv.end(), x);
    std::copy(zv.begin(), zv.end(), z);
    std::copy(rv.begin(), rv.end(), r);
}

std::int64_t ref_checksum(void *p, std::int64_t s0, std::int64_t s1) {
    return static_cast<RefHandle *>(p)->st->CheckSum(static_cast<int>(s0), static_cast<int>(s1));
}

const char *ref_backend(void *p) {
    static std::string name;
    name = static_cast<RefHandle *>(p)->st->GetKokkosBackend();
    return name.c_str();
}

// Test-only functors of the reference, driven on shot range [0, batch).
std::int32_t ref_row_product_sign(void *p, std::int64_t i, std::int64_t k) {
    auto *h = static_cast<RefHandle *>(p);
    Kokkos::View<int *> out("out", h->st->GetBatchSize());
    Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace> policy(0, h->st->GetBatchSize());
    Kokkos::parallel_for(policy, Plaquette::BatchRowProductSignFunctor<int>(h->st->GetX(), h->st->GetZ(),
                                                                              h->st->GetR(), out, i, k));
    return out(0);
}

void ref_row_multiply(void *p, std::int64_t i, std::int64_t k) {
    auto *h = static_cast<RefHandle *>(p);
    Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace> policy(0, h->st->GetBatchSize());
    Kokkos::parallel_for(policy,
                         Plaquette::BatchRowMultiplyFunctor<int>(h->st->GetX(), h->st->GetZ(), h->st->GetR(), i, k));
}

std::int32_t ref_measure_determined(void *p, std::int64_t q) {
    auto *h = static_cast<RefHandle *>(p);
    Kokkos::View<int *> out("out", h->st->GetBatchSize());
    Kokkos::RangePolicy<Kokkos::DefaultExecutionSpace> policy(0, h->st->GetBatchSize());
    Kokkos::parallel_for(policy, Plaquette::BatchMeasureDeterminedFunctor<int>(h->st->GetX(), h->st->GetZ(),
                                                                                 h->st->GetR(), out, q));
    return out(0);
}

std::int32_t ref_pauli_product_phase(std::int32_t x1, std::int32_t z1, std::int32_t x2, std::int32_t z2) {
    return Plaquette::PauliProductPhase<int>(x1, z1, x2, z2);
}

// Circuit replay with the same op encoding as ora_run.  Pauli channels take
// the oracle's outcomes (ora_channel_paulis: the reference has no channel op)
// and apply them through the reference's own flag gates.
int ref_run(void *p, const std::int32_t *ops, std::int64_t nops, const float *params, const std::uint8_t *forced_all) {
    auto *h = static_cast<RefHandle *>(p);
    const size_t B = h->st->GetBatchSize();
    const size_t fbytes = (B + 7) / 8;
    std::int64_t kmeas = 0;
    for (std::int64_t k = 0; k < nops; ++k) {
        const std::int32_t code = ops[4 * k], a = ops[4 * k + 1], b = ops[4 * k + 2], c = ops[4 * k + 3];
        const std::uint8_t *forced = forced_all ? forced_all + kmeas * fbytes : nullptr;
        switch (code) {
        case ORA_OP_H: h->st->ApplyHadamardGate(a); break;
        case ORA_OP_S: h->st->ApplyPhaseGate(a); break;
        case ORA_OP_X: h->st->ApplyPauliXGate(a); break;
        case ORA_OP_Y: h->st->ApplyPauliYGate(a); break;
        case ORA_OP_Z: h->st->ApplyPauliZGate(a); break;
        case ORA_OP_CX: h->st->ApplyControlNotGate(a, b); break;
        case ORA_OP_CZ: h->st->ApplyControlPhaseGate(a, b); break;
        case ORA_OP_M:
            ref_measure(p, a, c >= 0 ? params[c] : 0.5f, -1, forced);
            ++kmeas;
            break;
        case ORA_OP_R:
            ref_reset_qubit(p, a, forced);
            ++kmeas;
            break;
        case ORA_OP_PAULI1: {
            const std::uint64_t ev = h->events++;
            std::vector<int> fx(B), fz(B);
            std::vector<std::int32_t> pk(B + 1);
            ora_channel_paulis(h->seed, ev, h->shot_base, (std::int64_t)B, params + c, 3, pk.data());
            for (size_t s = 0; s < B; ++s) {
                int kk = pk[s];
                fx[s] = (kk == 1 || kk == 2);
                fz[s] = (kk == 2 || kk == 3);
            }
            cond_paulis(h, a, fx, fz);
            break;
        }
        case ORA_OP_PAULI2: {
            const std::uint64_t ev = h->events++;
            std::vector<int> fxa(B), fza(B), fxb(B), fzb(B);
            std::vector<std::int32_t> pk(B + 1);
            ora_channel_paulis(h->seed, ev, h->shot_base, (std::int64_t)B, params + c, 15, pk.data());
            for (size_t s = 0; s < B; ++s) {
                int kk = pk[s];
                int pa = kk >> 2, pb = kk & 3;
                fxa[s] = (pa == 1 || pa == 2);
                fza[s] = (pa == 2 || pa == 3);
                fxb[s] = (pb == 1 || pb == 2);
                fzb[s] = (pb == 2 || pb == 3);
            }
            cond_paulis(h, a, fxa, fza);
            cond_paulis(h, b, fxb, fzb);
            break;
        }
        case ORA_OP_H_IF: ref_h_flag(p, a, c); break;
        case ORA_OP_S_IF: ref_s_flag(p, a, c); break;
        default: return -1;
        }
    }
    return 0;
}

} // extern "C"
