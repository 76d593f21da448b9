// Serial stand-in for the parts of Kokkos that cajitafluids' own headers use,
// so that those headers (src/*.hpp) compile unchanged on the host for the
// oracle's reference pin.  TEST INFRASTRUCTURE ONLY: nothing in the product
// includes this directory.
//
// What it provides: Kokkos::Array, Kokkos::View<T***> (a reference-counted
// host array, zero-initialised, bounds-checked), the Serial execution space
// and HostSpace, parallel_for over a 2-D range (run in order), the
// KOKKOS_* function macros and no-op profiling regions.
#ifndef CFREF_KOKKOS_CORE_HPP
#define CFREF_KOKKOS_CORE_HPP

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_ENABLE_SERIAL 1

namespace Kokkos {

template <class T, std::size_t N>
struct Array {
    T m_data[N];
    T& operator[](std::size_t i) { return m_data[i]; }
    const T& operator[](std::size_t i) const { return m_data[i]; }
    T* data() { return m_data; }
    const T* data() const { return m_data; }
    static constexpr std::size_t size() { return N; }
};

struct Serial {};
struct HostSpace {};
template <class Exec, class Mem>
struct Device {
    using execution_space = Exec;
    using memory_space = Mem;
};

template <class DataType, class... Props>
class View;

// Rank-3 view (i, j, dof), i fastest.  Copies share the data, as Kokkos
// views do; every access is bounds-checked (an out-of-range index aborts
// with its coordinates instead of reading past the array).
template <class T, class... Props>
class View<T***, Props...> {
  public:
    View() = default;
    View(const std::string& label, std::size_t n0, std::size_t n1, std::size_t n2)
        : m_label(label), m_data(std::make_shared<std::vector<T>>(n0 * n1 * n2, T(0))), m_ext{n0, n1, n2} {}
    T& operator()(long i, long j, long k) const {
        if (i < 0 || j < 0 || k < 0 || (std::size_t)i >= m_ext[0] || (std::size_t)j >= m_ext[1] ||
            (std::size_t)k >= m_ext[2]) {
            std::fprintf(stderr, "View %s: index (%ld, %ld, %ld) outside (%zu, %zu, %zu)\n", m_label.c_str(), i, j,
                         k, m_ext[0], m_ext[1], m_ext[2]);
            std::abort();
        }
        return (*m_data)[((std::size_t)k * m_ext[1] + (std::size_t)j) * m_ext[0] + (std::size_t)i];
    }
    std::size_t extent(int d) const { return m_ext[d]; }
    T* data() const { return m_data ? m_data->data() : nullptr; }
    std::size_t size() const { return m_ext[0] * m_ext[1] * m_ext[2]; }

  private:
    std::string m_label;
    std::shared_ptr<std::vector<T>> m_data;
    std::size_t m_ext[3] = {0, 0, 0};
};

// A 2-D index range [lo, hi) per axis.
struct MDRangePolicy2 {
    long lo[2], hi[2];
};

// Runs f(i, j) over the range, j outer.  The kernels this runs write each
// index once and read only other arrays or their own index, so the order
// does not change their results.
template <class F>
void parallel_for(const std::string&, const MDRangePolicy2& p, const F& f) {
    for (long j = p.lo[1]; j < p.hi[1]; ++j)
        for (long i = p.lo[0]; i < p.hi[0]; ++i) f((int)i, (int)j);
}

namespace Profiling {
inline void pushRegion(const std::string&) {}
inline void popRegion() {}
}  // namespace Profiling

inline void fence() {}

}  // namespace Kokkos

#endif
