// Kokkos_Core.hpp -- minimal Kokkos-API shim (test infrastructure only).
//
// Written for this project from the documented semantics of the Kokkos API;
// no Kokkos source is used.  It implements exactly the API slice that the
// reference's headers use (plaquette_simulator/src/*.hpp): View (LayoutRight,
// host memory, reference-counted, optionally unmanaged), MDRangePolicy of
// rank 2/3, RangePolicy, parallel_for / parallel_reduce on OpenMP, deep_copy,
// initialize / finalize, and DefaultExecutionSpace::name().  With it the
// reference headers compile unmodified with g++ -fopenmp and serve as the
// pinned CPU oracle of the tableau path.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <optional>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION

namespace Kokkos {

struct HostSpace {
    static const char *name() { return "HostSpace"; }
};
struct OpenMP {
    static const char *name() { return "OpenMP"; }
};
using DefaultExecutionSpace = OpenMP;
using DefaultHostExecutionSpace = OpenMP;

enum : unsigned { Unmanaged = 1u };
template <unsigned Flags> struct MemoryTraits {
    static constexpr unsigned flags = Flags;
};

struct InitializationSettings {};

namespace shim {
inline bool &initialized_flag() {
    static bool v = false;
    return v;
}
inline bool &finalized_flag() {
    static bool v = false;
    return v;
}
// Index of the iteration the calling thread is executing inside a
// RangePolicy parallel_for (the shot index for the reference's
// measurement functor).  Read by the forced-outcome hook in Kokkos_Random.hpp.
inline thread_local std::int64_t current_index = 0;

template <class T> struct data_rank;
template <class T> struct data_rank<T *> {
    using value_type = T;
    static constexpr int rank = 1;
};
template <class T> struct data_rank<T **> {
    using value_type = T;
    static constexpr int rank = 2;
};
template <class T> struct data_rank<T ***> {
    using value_type = T;
    static constexpr int rank = 3;
};
} // namespace shim

inline void initialize(const InitializationSettings & = {}) {
    shim::initialized_flag() = true;
    shim::finalized_flag() = false;
}
inline void finalize() {
    shim::finalized_flag() = true;
    shim::initialized_flag() = false;
}
inline bool is_initialized() { return shim::initialized_flag(); }
inline bool is_finalized() { return shim::finalized_flag(); }

// Row-major (LayoutRight) host view of rank 1..3.
template <class DataType, class... Props> class View {
    using info = shim::data_rank<DataType>;

  public:
    using value_type = typename info::value_type;
    static constexpr int rank = info::rank;

    View() = default;

    template <class... Ext, class = std::enable_if_t<(sizeof...(Ext) == rank)>>
    View(const std::string &label, Ext... ext) : label_(label) {
        set_extents(static_cast<std::size_t>(ext)...);
        owner_ = std::shared_ptr<value_type[]>(new value_type[size() ? size() : 1]());
        data_ = owner_.get();
    }

    template <class... Ext, class = std::enable_if_t<(sizeof...(Ext) == rank)>>
    View(value_type *ptr, Ext... ext) : data_(ptr) {
        set_extents(static_cast<std::size_t>(ext)...);
    }

    template <class... P2> View(const View<DataType, P2...> &o) : label_(o.label()), data_(o.data()) {
        for (int k = 0; k < 3; ++k) ext_[k] = o.extent(k);
    }

    value_type &operator()(std::size_t i) const { return data_[i]; }
    value_type &operator()(std::size_t i, std::size_t j) const { return data_[i * ext_[1] + j]; }
    value_type &operator()(std::size_t i, std::size_t j, std::size_t k) const {
        return data_[(i * ext_[1] + j) * ext_[2] + k];
    }
    value_type &operator[](std::size_t i) const { return data_[i]; }

    std::size_t extent(int k) const { return k < rank ? ext_[k] : 1; }
    std::size_t size() const {
        std::size_t s = 1;
        for (int k = 0; k < rank; ++k) s *= ext_[k];
        return s;
    }
    value_type *data() const { return data_; }
    const std::string &label() const { return label_; }

  private:
    template <class... E> void set_extents(E... e) {
        std::size_t v[] = {e...};
        for (int k = 0; k < 3; ++k) ext_[k] = k < rank ? v[k] : 1;
    }
    std::string label_;
    std::shared_ptr<value_type[]> owner_;
    value_type *data_ = nullptr;
    std::size_t ext_[3] = {0, 0, 0};
};

template <class D1, class... P1, class D2, class... P2>
inline void deep_copy(const View<D1, P1...> &dst, const View<D2, P2...> &src) {
    if (dst.data() == src.data()) return;
    std::memcpy(dst.data(), src.data(), dst.size() * sizeof(typename View<D1, P1...>::value_type));
}

template <int N> struct Rank {
    static constexpr int rank = N;
};

template <class RankT> class MDRangePolicy {
  public:
    static constexpr int rank = RankT::rank;
    template <class LT, class UT> MDRangePolicy(const LT (&lo)[rank], const UT (&hi)[rank]) {
        for (int k = 0; k < rank; ++k) {
            lo_[k] = static_cast<std::int64_t>(lo[k]);
            hi_[k] = static_cast<std::int64_t>(hi[k]);
        }
    }
    std::int64_t lo_[3] = {0, 0, 0};
    std::int64_t hi_[3] = {1, 1, 1};
};

template <class ExecSpace = DefaultExecutionSpace> class RangePolicy {
  public:
    template <class B, class E>
    RangePolicy(B begin, E end) : begin_(static_cast<std::int64_t>(begin)), end_(static_cast<std::int64_t>(end)) {}
    std::int64_t begin_, end_;
};

template <class F> inline void parallel_for(const MDRangePolicy<Rank<2>> &p, const F &f) {
#pragma omp parallel for collapse(2) schedule(static)
    for (std::int64_t i = p.lo_[0]; i < p.hi_[0]; ++i)
        for (std::int64_t j = p.lo_[1]; j < p.hi_[1]; ++j) f(i, j);
}

template <class F> inline void parallel_for(const MDRangePolicy<Rank<3>> &p, const F &f) {
#pragma omp parallel for collapse(2) schedule(static)
    for (std::int64_t i = p.lo_[0]; i < p.hi_[0]; ++i)
        for (std::int64_t j = p.lo_[1]; j < p.hi_[1]; ++j)
            for (std::int64_t k = p.lo_[2]; k < p.hi_[2]; ++k) f(i, j, k);
}

template <class E, class F> inline void parallel_for(const RangePolicy<E> &p, const F &f) {
#pragma omp parallel for schedule(static)
    for (std::int64_t i = p.begin_; i < p.end_; ++i) {
        shim::current_index = i;
        f(i);
    }
}

template <class F, class T> inline void parallel_reduce(const MDRangePolicy<Rank<3>> &p, const F &f, T &result) {
    T total = 0;
#pragma omp parallel for collapse(2) schedule(static) reduction(+ : total)
    for (std::int64_t i = p.lo_[0]; i < p.hi_[0]; ++i)
        for (std::int64_t j = p.lo_[1]; j < p.hi_[1]; ++j) {
            T local = 0;
            for (std::int64_t k = p.lo_[2]; k < p.hi_[2]; ++k) f(i, j, k, local);
            total += local;
        }
    result = total;
}

inline void fence() {}

} // namespace Kokkos
