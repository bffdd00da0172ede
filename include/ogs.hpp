/*
 * ogs.hpp -- C++ drop-in for libParanumal's single-rank ogs::ogs_t, header-only
 * over the C ABI in ogs_c.h (link with libdawgs_ogs.so).
 *
 * Mirrors the reference interface (include/ogs.hpp:174-345 of paranumal/dawgs):
 * the same namespace (libp::ogs), enums (Type, Op, Transpose, Method, Kind),
 * class (ogs_t), member counts (N, Ngather, NgatherGlobal, NlocalT, NlocalP,
 * NhaloT, NhaloP, ogsBase.hpp:48-58) and methods (Setup, Free,
 * GatherScatter/Gather/Scatter with their Start/Finish pairs, host and device
 * overloads, SetupGlobalToLocalMapping).  Failures throw libp::exception, as
 * LIBP_ABORT does in the reference (include/utils.hpp:57-76).
 *
 * The buffer types are minimal stand-ins for the reference containers
 * (include/memory.hpp): memory<T> (host, shared ownership, offset arithmetic),
 * pinnedMemory<T> (page-locked host) and deviceMemory<T> (CUDA device).  When
 * built inside libParanumal, define OGS_GB300_EXTERNAL_CONTAINERS and include
 * the project's own memory.hpp/comm.hpp/platform.hpp first: the templates below
 * only need T* ptr() from each container and the CUDA stream of platform_t.
 *
 * comm_t, Method and platform_t are accepted and ignored beyond the stream:
 * the path runs at one rank, with no MPI exchange.
 */
#ifndef OGS_GB300_OGS_HPP
#define OGS_GB300_OGS_HPP

#include <cstdint>
#include <cstring>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>

#include <cuda_runtime.h>

#include "ogs_c.h"

namespace libp {

#ifndef OGS_GB300_EXTERNAL_CONTAINERS
typedef int dlong;             /* include/types.h:59-63 */
typedef long long int hlong;   /* include/types.h:52-56 */

class exception : public std::runtime_error {
 public:
  explicit exception(const std::string& what) : std::runtime_error(what) {}
};

/* host buffer: memory.hpp:34-276 subset */
template <typename T>
class memory {
 public:
  memory() = default;
  explicit memory(size_t n) { malloc(n); }
  memory(size_t n, const T& val) {
    malloc(n);
    for (size_t i = 0; i < n; ++i) ptr()[i] = val;
  }
  void malloc(size_t n) {
    data_ = std::shared_ptr<T[]>(new T[n ? n : 1]());
    n_ = n;
    off_ = 0;
  }
  void calloc(size_t n) { malloc(n); }
  void free() { data_.reset(); n_ = off_ = 0; }
  T* ptr() { return data_ ? data_.get() + off_ : nullptr; }
  const T* ptr() const { return data_ ? data_.get() + off_ : nullptr; }
  size_t length() const { return n_; }
  T& operator[](size_t i) { return ptr()[i]; }
  const T& operator[](size_t i) const { return ptr()[i]; }
  memory operator+(ptrdiff_t d) const {
    memory m(*this);
    m.off_ += d;
    m.n_ -= d;
    return m;
  }
  void copyFrom(const memory& src, size_t count = 0) {
    std::memcpy(ptr(), src.ptr(), (count ? count : n_) * sizeof(T));
  }
  void copyTo(memory& dst, size_t count = 0) const {
    std::memcpy(dst.ptr(), ptr(), (count ? count : n_) * sizeof(T));
  }

 private:
  std::shared_ptr<T[]> data_;
  size_t n_ = 0, off_ = 0;
};

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw exception(std::string(what) + ": " + cudaGetErrorString(e));
}

/* page-locked host buffer: memory.hpp:464-690 subset */
template <typename T>
class pinnedMemory {
 public:
  pinnedMemory() = default;
  explicit pinnedMemory(size_t n) { malloc(n); }
  void malloc(size_t n) {
    T* p = nullptr;
    cuda_check(cudaMallocHost(reinterpret_cast<void**>(&p), (n ? n : 1) * sizeof(T)), "cudaMallocHost");
    data_ = std::shared_ptr<T>(p, [](T* q) { cudaFreeHost(q); });
    n_ = n;
  }
  void free() { data_.reset(); n_ = 0; }
  T* ptr() { return data_.get(); }
  const T* ptr() const { return data_.get(); }
  size_t length() const { return n_; }
  T& operator[](size_t i) { return ptr()[i]; }

 private:
  std::shared_ptr<T> data_;
  size_t n_ = 0;
};

/* device buffer: memory.hpp:284-460 subset */
template <typename T>
class deviceMemory {
 public:
  deviceMemory() = default;
  explicit deviceMemory(size_t n) { malloc(n); }
  void malloc(size_t n) {
    T* p = nullptr;
    cuda_check(cudaMalloc(reinterpret_cast<void**>(&p), (n ? n : 1) * sizeof(T)), "cudaMalloc");
    data_ = std::shared_ptr<T>(p, [](T* q) { cudaFree(q); });
    n_ = n;
    off_ = 0;
  }
  void free() { data_.reset(); n_ = off_ = 0; }
  T* ptr() { return data_ ? data_.get() + off_ : nullptr; }
  const T* ptr() const { return data_ ? data_.get() + off_ : nullptr; }
  size_t length() const { return n_; }
  deviceMemory operator+(ptrdiff_t d) const {
    deviceMemory m(*this);
    m.off_ += d;
    m.n_ -= d;
    return m;
  }
  void copyFrom(const T* src, size_t count = 0) {
    cuda_check(cudaMemcpy(ptr(), src, (count ? count : n_) * sizeof(T), cudaMemcpyHostToDevice), "copyFrom");
  }
  void copyFrom(const memory<T>& src, size_t count = 0) { copyFrom(src.ptr(), count); }
  void copyTo(T* dst, size_t count = 0) const {
    cuda_check(cudaMemcpy(dst, ptr(), (count ? count : n_) * sizeof(T), cudaMemcpyDeviceToHost), "copyTo");
  }
  void copyTo(memory<T>& dst, size_t count = 0) const { copyTo(dst.ptr(), count); }

 private:
  std::shared_ptr<T> data_;
  size_t n_ = 0, off_ = 0;
};

/* single-rank stand-in for comm_t (include/comm.hpp:68-567) */
class comm_t {
 public:
  int rank() const { return 0; }
  int size() const { return 1; }
};

/* the part of platform_t (include/platform.hpp:56-188) the path uses: a stream */
class platform_t {
 public:
  cudaStream_t stream = nullptr;
  template <typename T>
  deviceMemory<T> malloc(size_t n) { return deviceMemory<T>(n); }
  template <typename T>
  deviceMemory<T> malloc(size_t n, const memory<T>& src) {
    deviceMemory<T> d(n);
    d.copyFrom(src, n);
    return d;
  }
  void finish() { cuda_check(cudaStreamSynchronize(stream), "platform finish"); }
};
#endif /* OGS_GB300_EXTERNAL_CONTAINERS */

namespace ogs {

typedef enum { Float, Double, Int32, Int64 } Type;        /* ogs.hpp:179 */
typedef enum { Add, Mul, Max, Min } Op;                   /* ogs.hpp:186 */
typedef enum { Sym, NoTrans, Trans } Transpose;           /* ogs.hpp:189 */
typedef enum { Auto, Pairwise, CrystalRouter, AllToAll } Method;  /* ogs.hpp:192 */
typedef enum { Unsigned, Signed, Halo } Kind;             /* ogs.hpp:195 */

template <typename T> struct ogsType;
template <> struct ogsType<float> { static constexpr Type get() { return Float; } };
template <> struct ogsType<double> { static constexpr Type get() { return Double; } };
template <> struct ogsType<int> { static constexpr Type get() { return Int32; } };
template <> struct ogsType<long long int> { static constexpr Type get() { return Int64; } };

/* ogs.hpp:213 -- the kernels are compiled ahead of time, nothing to build */
inline void InitializeKernels(platform_t&, const Type, const Op) {}

class ogs_t {
 public:
  dlong N = 0;
  dlong Ngather = 0;
  dlong NlocalT = 0, NhaloT = 0, NlocalP = 0, NhaloP = 0;
  hlong NgatherGlobal = 0;
  Kind kind = Unsigned;
  bool unique = false;
  bool gather_defined = false;

  ogs_t() = default;

  /* ogs.hpp:221-228, ogsSetup.cpp:44-53 */
  void Setup(const dlong _N, memory<hlong> ids, comm_t /*comm*/, const Kind _kind,
             const Method method, const bool _unique, const bool verbose, platform_t& platform) {
    Free();
    stream_ = platform.stream;
    static_assert(sizeof(hlong) == sizeof(int64_t), "hlong must be 64-bit");
    ogs_handle raw = nullptr;
    check(ogs_setup(&raw, _N, reinterpret_cast<int64_t*>(ids.ptr()), static_cast<int>(_kind),
                    static_cast<int>(method), _unique ? 1 : 0, verbose ? 1 : 0));
    hp_ = std::shared_ptr<ogs_handle_s>(raw, [](ogs_handle q) { ogs_free(q); });
    h_ = raw;
    ogs_counts c;
    check(ogs_get_counts(h_, &c));
    N = static_cast<dlong>(c.N);
    Ngather = static_cast<dlong>(c.Ngather);
    NlocalT = static_cast<dlong>(c.NlocalT);
    NlocalP = static_cast<dlong>(c.NlocalP);
    NgatherGlobal = c.NgatherGlobal;
    kind = _kind;
    unique = _unique;
    gather_defined = c.gather_defined != 0;
  }

  /* copies share the handle, like the reference's shared_ptr members
   * (ogsBase.hpp:80-82); the last one releases it */
  void Free() {
    hp_.reset();
    h_ = nullptr;
    N = Ngather = NlocalT = NlocalP = 0;
    NgatherGlobal = 0;
  }

  /* ogs_t::SetupGlobalToLocalMapping (ogsSetup.cpp:866-886): a NoTrans
   * scatter of the row numbers through the T maps, so GlobalToLocal[n] = row
   * of node n and -1 for nodes that take part in no row. */
  void SetupGlobalToLocalMapping(memory<dlong> GlobalToLocal) {
    std::unique_ptr<int32_t[]> rs(new int32_t[NlocalT + 1]);
    std::unique_ptr<int32_t[]> ci(new int32_t[N ? N : 1]);
    check(ogs_get_maps(h_, rs.get(), ci.get(), nullptr, nullptr));
    for (dlong n = 0; n < N; ++n) GlobalToLocal[n] = -1;
    for (dlong r = 0; r < NlocalT; ++r)
      for (int32_t j = rs[r]; j < rs[r + 1]; ++j) GlobalToLocal[ci[j]] = r;
  }

  /* ---- GatherScatter, ogs.hpp:232-265 ---- */
  template <typename T>
  void GatherScatter(memory<T> v, const int k, const Op op, const Transpose trans) {
    check(ogs_gather_scatter_host(h_, v.ptr(), k, ogsType<T>::get(), op, trans, stream_));
  }
  template <typename T>
  void GatherScatter(deviceMemory<T> o_v, const int k, const Op op, const Transpose trans) {
    check(ogs_gather_scatter(h_, o_v.ptr(), k, ogsType<T>::get(), op, trans, stream_));
  }
  template <typename V>
  void GatherScatterStart(V v, const int k, const Op op, const Transpose trans) {
    GatherScatter(v, k, op, trans);
  }
  template <typename V>
  void GatherScatterFinish(V, const int, const Op, const Transpose) {}

  /* ---- Gather, ogs.hpp:268-306 ---- */
  template <typename T>
  void Gather(memory<T> gv, const memory<T> v, const int k, const Op op, const Transpose trans) {
    check(ogs_gather_host(h_, gv.ptr(), v.ptr(), k, ogsType<T>::get(), op, trans, stream_));
  }
  template <typename T>
  void Gather(deviceMemory<T> o_gv, deviceMemory<T> o_v, const int k, const Op op, const Transpose trans) {
    check(ogs_gather(h_, o_gv.ptr(), o_v.ptr(), k, ogsType<T>::get(), op, trans, stream_));
  }
  template <typename G, typename V>
  void GatherStart(G gv, V v, const int k, const Op op, const Transpose trans) {
    Gather(gv, v, k, op, trans);
  }
  template <typename G, typename V>
  void GatherFinish(G, V, const int, const Op, const Transpose) {}

  /* ---- Scatter, ogs.hpp:309-341 ---- */
  template <typename T>
  void Scatter(memory<T> v, const memory<T> gv, const int k, const Transpose trans) {
    check(ogs_scatter_host(h_, v.ptr(), gv.ptr(), k, ogsType<T>::get(), trans, stream_));
  }
  template <typename T>
  void Scatter(deviceMemory<T> o_v, deviceMemory<T> o_gv, const int k, const Transpose trans) {
    check(ogs_scatter(h_, o_v.ptr(), o_gv.ptr(), k, ogsType<T>::get(), trans, stream_));
  }
  template <typename V, typename G>
  void ScatterStart(V v, G gv, const int k, const Transpose trans) {
    Scatter(v, gv, k, trans);
  }
  template <typename V, typename G>
  void ScatterFinish(V, G, const int, const Transpose) {}

  /* No reference counterpart: reserve the staging of the host-buffer
   * (memory<T>) overloads for k components of T, so that later calls of no
   * larger size allocate nothing (ogs_reserve_host). */
  template <typename T>
  void ReserveHost(const int k) {
    check(ogs_reserve_host(h_, k, ogsType<T>::get()));
  }

  ogs_handle handle() const { return h_; }

 private:
  static void check(ogs_status s) {
    if (s != OGS_OK) {
      std::ostringstream os;
      os << "ogs error " << static_cast<int>(s) << ": " << ogs_last_error_string();
      throw exception(os.str());
    }
  }
  std::shared_ptr<ogs_handle_s> hp_;
  ogs_handle h_ = nullptr;
  cudaStream_t stream_ = nullptr;
};

/* halo_t (include/ogs.hpp:346-397 of the reference; libs/ogs/ogsHalo.cpp).
 * Setup at one rank checks the ids and has no halo rows; SetupFromGather
 * takes its counts from an ogs_t.  A multi-rank caller attaches its exchange
 * (the MPI step) with SetExchange and builds the halo from its gatherHalo maps
 * through ogs_halo_setup_maps (see ogs_c.h). */
class halo_t {
 public:
  bool gathered_halo = false;
  dlong N = 0, Nhalo = 0, NlocalT = 0, NhaloP = 0, NhaloT = 0;

  halo_t() = default;

  /* ogsSetup.cpp:55-64 */
  void Setup(const dlong _N, memory<hlong> ids, comm_t /*comm*/, const Method method, const bool verbose,
             platform_t& platform) {
    ogs_halo raw = nullptr;
    check(ogs_halo_setup(&raw, _N, reinterpret_cast<const int64_t*>(ids.ptr()), static_cast<int>(method),
                         verbose ? 1 : 0));
    adopt(raw, platform.stream);
  }
  /* ogsSetup.cpp:888-913 */
  void SetupFromGather(ogs_t& ogs) {
    if (!ogs.gather_defined) throw exception("Gather operation not well-defined.");
    ogs_halo raw = nullptr;
    check(ogs_halo_setup_from_gather(&raw, ogs.NlocalT, ogs.NhaloP, ogs.NhaloT, 0));
    adopt(raw, stream_);
  }
  /* no reference counterpart: the exchange (MPI) step of a multi-rank caller */
  void SetExchange(const ogs_exchange& x) {
    x_ = x;
    has_x_ = true;
  }
  void Free() {
    hp_.reset();
    h_ = nullptr;
    N = Nhalo = NlocalT = NhaloP = NhaloT = 0;
  }

  template <typename T>
  void Exchange(memory<T> v, const int k) {
    check(ogs_halo_exchange_host(h_, v.ptr(), k, ogs::ogsType<T>::get(), xp(), stream_));
  }
  template <typename T>
  void Exchange(deviceMemory<T> o_v, const int k) {
    check(ogs_halo_exchange(h_, o_v.ptr(), k, ogs::ogsType<T>::get(), xp(), stream_));
  }
  template <typename T>
  void ExchangeStart(deviceMemory<T> o_v, const int k) {
    check(ogs_halo_exchange_start(h_, o_v.ptr(), k, ogs::ogsType<T>::get(), xp(), stream_));
  }
  template <typename T>
  void ExchangeFinish(deviceMemory<T> o_v, const int k) {
    check(ogs_halo_exchange_finish(h_, o_v.ptr(), k, ogs::ogsType<T>::get(), xp(), stream_));
  }
  template <typename T>
  void ExchangeStart(memory<T> v, const int k) { Exchange(v, k); }
  template <typename T>
  void ExchangeFinish(memory<T>, const int) {}

  template <typename T>
  void Combine(memory<T> v, const int k) {
    check(ogs_halo_combine_host(h_, v.ptr(), k, ogs::ogsType<T>::get(), xp(), stream_));
  }
  template <typename T>
  void Combine(deviceMemory<T> o_v, const int k) {
    check(ogs_halo_combine(h_, o_v.ptr(), k, ogs::ogsType<T>::get(), xp(), stream_));
  }
  template <typename T>
  void CombineStart(deviceMemory<T> o_v, const int k) {
    check(ogs_halo_combine_start(h_, o_v.ptr(), k, ogs::ogsType<T>::get(), xp(), stream_));
  }
  template <typename T>
  void CombineFinish(deviceMemory<T> o_v, const int k) {
    check(ogs_halo_combine_finish(h_, o_v.ptr(), k, ogs::ogsType<T>::get(), xp(), stream_));
  }
  template <typename T>
  void CombineStart(memory<T> v, const int k) { Combine(v, k); }
  template <typename T>
  void CombineFinish(memory<T>, const int) {}

  ogs_halo handle() const { return h_; }

 private:
  void adopt(ogs_halo raw, cudaStream_t stream) {
    hp_ = std::shared_ptr<ogs_halo_s>(raw, [](ogs_halo q) { ogs_halo_free(q); });
    h_ = raw;
    stream_ = stream;
    ogs_halo_counts c;
    check(ogs_halo_get_counts(h_, &c));
    N = static_cast<dlong>(c.N);
    Nhalo = static_cast<dlong>(c.Nhalo);
    NlocalT = static_cast<dlong>(c.NlocalT);
    NhaloP = static_cast<dlong>(c.NhaloP);
    NhaloT = static_cast<dlong>(c.NhaloT);
    gathered_halo = c.gathered != 0;
  }
  const ogs_exchange* xp() const { return has_x_ ? &x_ : nullptr; }
  static void check(ogs_status s) {
    if (s != OGS_OK) {
      std::ostringstream os;
      os << "ogs error " << static_cast<int>(s) << ": " << ogs_last_error_string();
      throw exception(os.str());
    }
  }
  std::shared_ptr<ogs_halo_s> hp_;
  ogs_halo h_ = nullptr;
  cudaStream_t stream_ = nullptr;
  ogs_exchange x_{};
  bool has_x_ = false;
};

}  // namespace ogs
}  // namespace libp

#endif /* OGS_GB300_OGS_HPP */
