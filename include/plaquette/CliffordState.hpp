// plaquette/CliffordState.hpp -- C++ drop-in for the reference's
// Plaquette::CliffordState<Precision> (plaquette_simulator/src/CliffordState.hpp),
// header-only over the C ABI of libps_gpu.so (include/plaquette_gpu.h).
//
// Same class name, constructors and member functions as the reference, so
// code written against the reference compiles against this header with
//   #include <plaquette/CliffordState.hpp>   and   -lps_gpu.
// Differences: Kokkos Views are replaced by small views of the library's
// device memory.  A record's device array (Measurement::
// measurement_results_device) is a RecordView: the record id and its packed
// device words, which Apply*GateWithApplyFlag takes as the reference takes
// the View (or the record id itself).  GetX/GetZ/GetR give DeviceViews of
// the bit-packed planes ([2n+1][n][words] / [2n+1][words] uint64, bit s of
// word k = shot 64k + s) instead of int32 [batch][2n+1][n] Views; they feed
// DeviceToDevice as in the reference's copy constructor.  DeviceToHost
// still gives the reference layout.
#pragma once

#include <cstdint>
#include <deque>
#include <memory>
#include <optional>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../plaquette_gpu.h"

namespace Plaquette {

// Error.hpp:52-77: the exception type the reference throws.
class Exception : public std::exception {
  public:
    explicit Exception(const std::string &err_msg) noexcept : err_msg(err_msg) {}
    const char *what() const noexcept override { return err_msg.c_str(); }

  private:
    std::string err_msg;
};

namespace detail {
inline void check(ps_status st) {
    if (st != PS_OK) throw Exception(ps_last_error());
}
}  // namespace detail

// A measurement record's device array: its id in the state and its packed
// words (the reference passes Kokkos::View<Precision *> here).
struct RecordView {
    size_t id = 0;
    void *words = nullptr;
    size_t size = 0;  // shots
    size_t extent(size_t) const { return size; }
    void *data() const { return words; }
};

// A bit-packed device plane of a state (GetX / GetZ / GetR).
struct DeviceView {
    ps_state *owner = nullptr;
    void *data = nullptr;
    size_t rows = 0, cols = 0, words = 0;  // cols = 1 for R
};

template <class Precision> class CliffordState {
  public:
    // CliffordState.hpp:32-58: one measurement's records, host copies on
    // demand.  CopyToHost always reads the record again (a record measured
    // into again is never served stale).
    struct Measurement {
        size_t qubit_measured = 0;
        std::vector<Precision> measurement_results_host;
        std::vector<Precision> measurement_determined_host;
        std::unique_ptr<RecordView> measurement_results_device;
        std::unique_ptr<RecordView> measurement_determined_device;

        void CopyToHost() {
            const size_t S = measurement_results_device->size, nb = (S + 7) / 8;
            std::vector<uint8_t> res(nb), det(nb);
            detail::check(ps_get_record_bits(owner, measurement_results_device->id, res.data(), det.data()));
            measurement_results_host.resize(S);
            measurement_determined_host.resize(S);
            for (size_t s = 0; s < S; ++s) {
                measurement_results_host[s] = static_cast<Precision>((res[s >> 3] >> (s & 7)) & 1u);
                measurement_determined_host[s] = static_cast<Precision>((det[s >> 3] >> (s & 7)) & 1u);
            }
        }
        ps_state *owner = nullptr;
    };

    CliffordState() = delete;

    // CliffordState.hpp:97-139
    CliffordState(size_t num_qubits, size_t batch_size, int seed = -1, bool init_to_zero_state = true) {
        detail::check(ps_create(num_qubits, batch_size, seed, init_to_zero_state ? 1 : 0, &h_));
    }

    // CliffordState.hpp:153-159
    CliffordState(std::vector<Precision> &x, std::vector<Precision> &z, std::vector<Precision> &r,
                  size_t num_qubits, size_t batch_size, long int seed = -1) {
        const auto xi = to_int32(x), zi = to_int32(z), ri = to_int32(r);
        detail::check(ps_create_from_host(xi.data(), zi.data(), ri.data(), num_qubits, batch_size, seed, &h_));
    }

    // CliffordState.hpp:168-174 (records are not copied, as in the reference)
    CliffordState(const CliffordState &other) { detail::check(ps_clone(other.h_, &h_)); }
    CliffordState &operator=(const CliffordState &) = delete;
    CliffordState(CliffordState &&o) noexcept : h_(o.h_), measurements_(std::move(o.measurements_)) { o.h_ = nullptr; }

    ~CliffordState() { ps_destroy(h_); }

    // CliffordState.hpp:207-259, reference layout [batch][2n+1][n] / [batch][2n+1]
    void HostToDevice(std::vector<Precision> &x, std::vector<Precision> &z, std::vector<Precision> &r) {
        const auto xi = to_int32(x), zi = to_int32(z), ri = to_int32(r);
        detail::check(ps_host_to_device(h_, xi.data(), zi.data(), ri.data()));
    }

    auto DeviceToHost() {
        const size_t n = GetNumQubits(), B = GetBatchSize(), W = 2 * n + 1;
        std::vector<int32_t> x(B * W * n), z(B * W * n), r(B * W);
        detail::check(ps_device_to_host(h_, x.data(), z.data(), r.data()));
        return std::make_tuple(std::vector<Precision>(x.begin(), x.end()), std::vector<Precision>(z.begin(), z.end()),
                               std::vector<Precision>(r.begin(), r.end()));
    }

    std::string GetKokkosBackend() const { return ps_backend_name(); }  // :280-282

    size_t GetNumQubits() const {
        uint64_t v = 0;
        detail::check(ps_get_num_qubits(h_, &v));
        return v;
    }
    size_t GetBatchSize() const {
        uint64_t v = 0;
        detail::check(ps_get_batch_size(h_, &v));
        return v;
    }
    long int GetSeed() const {
        int64_t v = 0;
        detail::check(ps_get_seed(h_, &v));
        return v;
    }

    void ResetCliffordState() { detail::check(ps_reset(h_)); }  // :309-316

    Precision CheckSum(int starting_batch_id = 0, int ending_batch_id = -1) {  // :327-338
        int64_t v = 0;
        detail::check(ps_checksum(h_, starting_batch_id, ending_batch_id, &v));
        return static_cast<Precision>(v);
    }

    // :348-372, flag = the results of measurement record `measurement_id`
    void ApplyHadamardGateWithApplyFlag(size_t target_qubit, size_t measurement_id) {
        detail::check(ps_h_flag(h_, target_qubit, measurement_id));
    }
    void ApplyPhaseGateWithApplyFlag(size_t target_qubit, size_t measurement_id) {
        detail::check(ps_s_flag(h_, target_qubit, measurement_id));
    }
    // ... and as the reference calls them, with the record's device array
    // (*GetMeasurement(id).measurement_results_device)
    void ApplyHadamardGateWithApplyFlag(size_t target_qubit, const RecordView &flag) {
        ApplyHadamardGateWithApplyFlag(target_qubit, flag.id);
    }
    void ApplyPhaseGateWithApplyFlag(size_t target_qubit, const RecordView &flag) {
        ApplyPhaseGateWithApplyFlag(target_qubit, flag.id);
    }

    // :180-198: the packed device planes
    DeviceView GetX() const { return plane(0); }
    DeviceView GetZ() const { return plane(1); }
    DeviceView GetR() const { return plane(2); }

    // :268-274: copies another state's planes (same qubits and shots) into
    // this one, after that state's queued work.
    void DeviceToDevice(const DeviceView &x, const DeviceView &z, const DeviceView &r) {
        const DeviceView mine = plane(0);
        if (x.rows != mine.rows || x.cols != mine.cols || x.words != mine.words || z.words != mine.words ||
            r.rows != mine.rows || r.words != mine.words)
            throw Exception("DeviceToDevice: the planes belong to a state of another size");
        for (ps_state *o : {x.owner, z.owner, r.owner})
            if (o) detail::check(ps_synchronize(o));
        detail::check(ps_device_to_device(h_, x.data, z.data, r.data));
    }

    // :379-531
    void ApplyHadamardGateToQubits(const std::vector<size_t> &t) { apply(PS_OP_H, t); }
    void ApplyHadamardGate(size_t q) { detail::check(ps_h(h_, q)); }
    void ApplyControlNotGateToQubits(const std::vector<size_t> &t) { apply(PS_OP_CX, t); }
    void ApplyControlNotGate(size_t c, size_t t) { detail::check(ps_cx(h_, c, t)); }
    void ApplyControlPhaseGateToQubits(const std::vector<size_t> &t) { apply(PS_OP_CZ, t); }
    void ApplyControlPhaseGate(size_t c, size_t t) { detail::check(ps_cz(h_, c, t)); }
    void ApplyPhaseGateToQubits(const std::vector<size_t> &t) { apply(PS_OP_S, t); }
    void ApplyPhaseGate(size_t q) { detail::check(ps_s(h_, q)); }
    void ApplyPauliXGateToQubits(const std::vector<size_t> &t) { apply(PS_OP_X, t); }
    void ApplyPauliXGate(size_t q) { detail::check(ps_x(h_, q)); }
    void ApplyPauliYGateToQubits(const std::vector<size_t> &t) { apply(PS_OP_Y, t); }
    void ApplyPauliYGate(size_t q) { detail::check(ps_y(h_, q)); }
    void ApplyPauliZGateToQubits(const std::vector<size_t> &t) { apply(PS_OP_Z, t); }
    void ApplyPauliZGate(size_t q) { detail::check(ps_z(h_, q)); }

    // :543-548
    void MeasureQubits(const std::vector<size_t> &targets, float bias = 0.5) {
        for (size_t q : targets) MeasureQubit(q, bias);
    }

    // :587-623
    size_t MeasureQubit(size_t target_qubit, float bias = 0.5, std::optional<size_t> measurement_id = std::nullopt) {
        uint64_t id = 0;
        const int64_t want = measurement_id ? static_cast<int64_t>(*measurement_id) : -1;
        detail::check(ps_measure(h_, target_qubit, bias, want, nullptr, &id));
        return id;
    }

    // :635-648
    std::optional<std::pair<int, int>> GetMeasurement(size_t measurement_id, size_t batch_index) {
        int32_t res = 0, det = 0;
        const ps_status st = ps_get_measurement(h_, measurement_id, batch_index, &res, &det);
        if (st == PS_E_RANGE) return std::nullopt;
        detail::check(st);
        return std::make_pair(static_cast<int>(res), static_cast<int>(det));
    }

    // :655-659: the record itself (host copies on demand, device arrays)
    Measurement &GetMeasurement(size_t measurement_id) {
        uint64_t nrec = 0;
        detail::check(ps_num_records(h_, &nrec));
        if (measurement_id >= nrec) throw Exception("Measurement id or batch index is out of range.");
        while (measurements_.size() <= measurement_id) {
            const size_t id = measurements_.size();
            Measurement m;
            uint64_t q = 0;
            void *res = nullptr, *det = nullptr;
            detail::check(ps_record_qubit(h_, id, &q));
            detail::check(ps_get_record_device(h_, id, &res, &det));
            m.owner = h_;
            m.qubit_measured = q;
            m.measurement_results_device.reset(new RecordView{id, res, GetBatchSize()});
            m.measurement_determined_device.reset(new RecordView{id, det, GetBatchSize()});
            measurements_.push_back(std::move(m));
        }
        return measurements_[measurement_id];
    }

    ps_state *handle() const { return h_; }

  private:
    DeviceView plane(int k) const {
        void *p[3] = {nullptr, nullptr, nullptr};
        uint64_t words = 0;
        detail::check(ps_get_device_tableau(h_, &p[0], &p[1], &p[2], &words));
        const size_t n = GetNumQubits();
        return DeviceView{h_, p[k], 2 * n + 1, k == 2 ? size_t(1) : n, static_cast<size_t>(words)};
    }

    template <class V> static std::vector<int32_t> to_int32(const V &v) { return std::vector<int32_t>(v.begin(), v.end()); }

    void apply(int32_t code, const std::vector<size_t> &t) {
        std::vector<uint64_t> u(t.begin(), t.end());
        detail::check(ps_apply_to_qubits(h_, code, u.data(), u.size()));
    }

    ps_state *h_ = nullptr;
    std::deque<Measurement> measurements_;  // GetMeasurement(id) entries (references stay valid)
};

}  // namespace Plaquette
