// Host-only stand-in for the subset of Kokkos that the reference's src/
// uses, so that those sources compile unmodified into a CPU program here
// (test infrastructure: the reference's own arithmetic, run as a checker
// for the oracle and as the timed CPU baseline).  It is not Kokkos.
//
// What the reference needs (src/lbm.hpp:26-110, src/lbm.cpp,
// src/mpi_view_transfer.cpp):
//   View<T*..., LayoutRight, Space>   reference-counted arrays of rank 1-4,
//                                     zero-initialised, index (i, j, k, l)
//                                     with the last index fastest
//   subview(v, ALL | pair...)         strided windows of a View
//   deep_copy([exec,] dst, src)       element-wise copy of equal extents
//   create_mirror_view(HostSpace, v)  v itself (everything is host memory)
//   parallel_for / parallel_reduce    over MDRangePolicy<Rank<3|4>>, run
//                                     with OpenMP threads; reductions with
//                                     Sum / Max / Min reducers, combined in
//                                     thread order (deterministic for a
//                                     fixed thread count)
//   fence, initialize, finalize       no-ops: every call above is
//                                     synchronous
// Threads per parallel region: imexref_threads() (shim_mpi.cpp), so that
// several ranks run as threads of one process without oversubscribing.
#pragma once

#include <cfloat>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include <omp.h>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [ =, *this ]

int imexref_threads();  // OpenMP threads per parallel region of this rank

namespace Kokkos {

struct HostSpace {};
struct LayoutRight {};
struct LayoutStride {};

struct OpenMP {
    using memory_space = HostSpace;
    void fence() const {}
};
using DefaultExecutionSpace = OpenMP;
using DefaultHostExecutionSpace = OpenMP;

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}
inline void fence() {}

struct ALL_t {};
constexpr ALL_t ALL{};

namespace detail {
template <class T>
struct rank_of {
    static constexpr int value = 0;
    using type = T;
};
template <class T>
struct rank_of<T*> {
    static constexpr int value = 1 + rank_of<T>::value;
    using type = typename rank_of<T>::type;
};
}  // namespace detail

template <class DataType, class... Props>
class View {
   public:
    static constexpr int R = detail::rank_of<DataType>::value;
    using value_type = typename detail::rank_of<DataType>::type;
    static_assert(R >= 1 && R <= 4, "shim Views have rank 1 to 4");

    View() = default;

    template <class... N, class = std::enable_if_t<sizeof...(N) == R>>
    View(const std::string& label, N... n) : label_(label)
    {
        const size_t ext[R] = {static_cast<size_t>(n)...};
        size_t total = 1;
        for (int r = R - 1; r >= 0; --r) {
            ext_[r] = ext[r];
            stride_[r] = total;
            total *= ext[r];
        }
        size_ = total;
        store_ = std::shared_ptr<value_type>(new value_type[total ? total : 1](), std::default_delete<value_type[]>());
        data_ = store_.get();
    }

    value_type* data() const { return data_; }
    size_t size() const { return size_; }
    size_t extent(int r) const { return r < R ? ext_[r] : 1; }
    int64_t extent_int(int r) const { return (int64_t)extent(r); }
    size_t stride(int r) const { return stride_[r]; }
    const std::string& label() const { return label_; }
    bool contiguous() const
    {
        size_t s = 1;
        for (int r = R - 1; r >= 0; --r) {
            if (ext_[r] > 1 && stride_[r] != s) return false;
            s *= ext_[r];
        }
        return true;
    }

    value_type& operator()(int64_t i) const { return data_[i * stride_[0]]; }
    value_type& operator()(int64_t i, int64_t j) const { return data_[i * stride_[0] + j * stride_[1]]; }
    value_type& operator()(int64_t i, int64_t j, int64_t k) const
    {
        return data_[i * stride_[0] + j * stride_[1] + k * stride_[2]];
    }
    value_type& operator()(int64_t i, int64_t j, int64_t k, int64_t l) const
    {
        return data_[i * stride_[0] + j * stride_[1] + k * stride_[2] + l * stride_[3]];
    }

    // a window: the same storage, offset and cut per dimension
    View window(const size_t (&lo)[4], const size_t (&hi)[4]) const
    {
        View v = *this;
        size_t off = 0, total = 1;
        for (int r = 0; r < R; ++r) {
            if (hi[r] < lo[r] || hi[r] > ext_[r]) throw std::out_of_range("subview out of range: " + label_);
            off += lo[r] * stride_[r];
            v.ext_[r] = hi[r] - lo[r];
            total *= v.ext_[r];
        }
        v.data_ = data_ + off;
        v.size_ = total;
        return v;
    }

   private:
    std::string label_;
    std::shared_ptr<value_type> store_;
    value_type* data_ = nullptr;
    size_t ext_[4] = {1, 1, 1, 1};
    size_t stride_[4] = {0, 0, 0, 0};
    size_t size_ = 0;
};

namespace detail {
inline void bounds(const ALL_t&, size_t ext, size_t& lo, size_t& hi)
{
    lo = 0;
    hi = ext;
}
template <class A, class B>
inline void bounds(const std::pair<A, B>& p, size_t, size_t& lo, size_t& hi)
{
    lo = (size_t)p.first;
    hi = (size_t)p.second;
}
}  // namespace detail

template <class D, class... P, class... S>
View<D, P...> subview(const View<D, P...>& v, const S&... s)
{
    static_assert(sizeof...(S) == View<D, P...>::R, "subview takes one range per dimension");
    size_t lo[4] = {0, 0, 0, 0}, hi[4] = {1, 1, 1, 1};
    int r = 0;
    ((detail::bounds(s, v.extent(r), lo[r], hi[r]), ++r), ...);
    return v.window(lo, hi);
}

template <class V>
V create_mirror_view(const HostSpace&, const V& v)
{
    return v;
}
template <class V>
V create_mirror_view(const V& v)
{
    return v;
}

template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src)
{
    constexpr int R = View<D1, P1...>::R;
    static_assert(R == View<D2, P2...>::R, "deep_copy between Views of different rank");
    for (int r = 0; r < R; ++r)
        if (dst.extent(r) != src.extent(r)) throw std::runtime_error("deep_copy: extents differ: " + dst.label());
    if (dst.data() == src.data()) return;
    const int64_t n0 = dst.extent_int(0), n1 = dst.extent_int(1), n2 = dst.extent_int(2), n3 = dst.extent_int(3);
    auto* d = dst.data();
    const auto* s = src.data();
    const size_t ds[4] = {dst.stride(0), R > 1 ? dst.stride(1) : 0, R > 2 ? dst.stride(2) : 0, R > 3 ? dst.stride(3) : 0};
    const size_t ss[4] = {src.stride(0), R > 1 ? src.stride(1) : 0, R > 2 ? src.stride(2) : 0, R > 3 ? src.stride(3) : 0};
#pragma omp parallel for collapse(2) schedule(static) num_threads(imexref_threads())
    for (int64_t a = 0; a < n0; ++a)
        for (int64_t b = 0; b < n1; ++b)
            for (int64_t c = 0; c < n2; ++c)
                for (int64_t e = 0; e < n3; ++e)
                    d[a * ds[0] + b * ds[1] + c * ds[2] + e * ds[3]] = s[a * ss[0] + b * ss[1] + c * ss[2] + e * ss[3]];
}

template <class Ex, class D1, class... P1, class D2, class... P2>
void deep_copy(const Ex&, const View<D1, P1...>& dst, const View<D2, P2...>& src)
{
    deep_copy(dst, src);
}

// ------------------------------------------------------------- policies --

enum class Iterate { Default, Left, Right };

template <unsigned N, Iterate Outer = Iterate::Default, Iterate Inner = Iterate::Default>
struct Rank {
    static constexpr int rank = (int)N;
};

template <unsigned MaxThreads = 0, unsigned MinBlocks = 0>
struct LaunchBounds {};

namespace detail {
template <class... P>
struct rank_in;
template <>
struct rank_in<> {
    static constexpr int value = 0;
};
template <unsigned N, Iterate O, Iterate I, class... P>
struct rank_in<Rank<N, O, I>, P...> {
    static constexpr int value = (int)N;
};
template <class A, class... P>
struct rank_in<A, P...> {
    static constexpr int value = rank_in<P...>::value;
};
}  // namespace detail

template <class... P>
struct MDRangePolicy {
    static constexpr int R = detail::rank_in<P...>::value;
    int64_t lo[4] = {0, 0, 0, 0}, hi[4] = {1, 1, 1, 1};
    MDRangePolicy(std::initializer_list<int64_t> b, std::initializer_list<int64_t> e,
                  std::initializer_list<int64_t> /*tile*/ = {})
    {
        if ((int)b.size() != R || (int)e.size() != R) throw std::runtime_error("MDRangePolicy: rank mismatch");
        int r = 0;
        for (int64_t v : b) lo[r++] = v;
        r = 0;
        for (int64_t v : e) hi[r++] = v;
    }
};

template <class... P>
struct RangePolicy {
    int64_t lo = 0, hi = 0;
    RangePolicy() = default;
    RangePolicy(int64_t b, int64_t e) : lo(b), hi(e) {}
};

template <class... P>
struct TeamPolicy {
    struct member_type {};
};

template <class... P, class F>
void parallel_for(const std::string&, const MDRangePolicy<P...>& p, const F& f)
{
    constexpr int R = MDRangePolicy<P...>::R;
    static_assert(R == 3 || R == 4, "shim parallel_for: MDRange rank 3 or 4");
    if constexpr (R == 3) {
#pragma omp parallel for collapse(2) schedule(static) num_threads(imexref_threads())
        for (int64_t i = p.lo[0]; i < p.hi[0]; ++i)
            for (int64_t j = p.lo[1]; j < p.hi[1]; ++j)
                for (int64_t k = p.lo[2]; k < p.hi[2]; ++k) f((int)i, (int)j, (int)k);
    } else {
#pragma omp parallel for collapse(2) schedule(static) num_threads(imexref_threads())
        for (int64_t a = p.lo[0]; a < p.hi[0]; ++a)
            for (int64_t i = p.lo[1]; i < p.hi[1]; ++i)
                for (int64_t j = p.lo[2]; j < p.hi[2]; ++j)
                    for (int64_t k = p.lo[3]; k < p.hi[3]; ++k) f((int)a, (int)i, (int)j, (int)k);
    }
}

template <class... P, class F>
void parallel_for(const std::string&, const RangePolicy<P...>& p, const F& f)
{
#pragma omp parallel for schedule(static) num_threads(imexref_threads())
    for (int64_t i = p.lo; i < p.hi; ++i) f((int)i);
}

// ------------------------------------------------------------- reducers --

template <class T>
struct Sum {
    using value_type = T;
    T& ref;
    explicit Sum(T& r) : ref(r) {}
    static T identity() { return T(0); }
    static void join(T& a, const T& b) { a += b; }
};

template <class T>
struct Max {
    using value_type = T;
    T& ref;
    explicit Max(T& r) : ref(r) {}
    static T identity() { return -DBL_MAX; }
    static void join(T& a, const T& b)
    {
        if (b > a) a = b;
    }
};

template <class T>
struct Min {
    using value_type = T;
    T& ref;
    explicit Min(T& r) : ref(r) {}
    static T identity() { return DBL_MAX; }
    static void join(T& a, const T& b)
    {
        if (b < a) a = b;
    }
};

namespace detail {
template <class Tup, class Red, size_t... I>
void join_all(Tup& a, const Tup& b, std::index_sequence<I...>)
{
    (std::tuple_element_t<I, Red>::join(std::get<I>(a), std::get<I>(b)), ...);
}
template <class Tup, class Red, size_t... I>
void store_all(const Tup& v, Red& reds, std::index_sequence<I...>)
{
    ((std::get<I>(reds).ref = std::get<I>(v)), ...);
}
}  // namespace detail

// Each thread folds its static share of the range into its own values
// (starting at the reducers' identities); the threads' values are then
// joined in thread order.
template <class... P, class F, class... Red>
void parallel_reduce(const std::string&, const MDRangePolicy<P...>& p, const F& f, Red... reds)
{
    static_assert(MDRangePolicy<P...>::R == 3, "shim parallel_reduce: MDRange rank 3");
    using Vals = std::tuple<typename Red::value_type...>;
    using Reds = std::tuple<Red...>;
    const int nt = imexref_threads();
    std::vector<Vals> part((size_t)nt, Vals(Red::identity()...));
#pragma omp parallel num_threads(nt)
    {
        Vals loc(Red::identity()...);
#pragma omp for collapse(2) schedule(static)
        for (int64_t i = p.lo[0]; i < p.hi[0]; ++i)
            for (int64_t j = p.lo[1]; j < p.hi[1]; ++j)
                for (int64_t k = p.lo[2]; k < p.hi[2]; ++k)
                    std::apply([&](auto&... v) { f((int)i, (int)j, (int)k, v...); }, loc);
        part[(size_t)omp_get_thread_num()] = loc;
    }
    Vals tot(Red::identity()...);
    for (const Vals& v : part) detail::join_all<Vals, Reds>(tot, v, std::index_sequence_for<Red...>{});
    Reds r(reds...);
    detail::store_all(tot, r, std::index_sequence_for<Red...>{});
}

}  // namespace Kokkos
