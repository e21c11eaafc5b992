// Shared host/device infrastructure of the sm_103a spatial-join library:
// status handling, the caller-supplied allocator, and small device helpers.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <type_traits>
#include <utility>

#include "../../include/cuspatial_gb300.h"

namespace cspt {

// ---------------------------------------------------------------------------
// errors: the reference throws cuspatial::logic_error (CUSPATIAL_EXPECTS,
// cpp/include/cuspatial/error.hpp:76) and cuspatial::cuda_error
// (CUSPATIAL_CUDA_TRY, error.hpp:143); here they become a status plus a
// per-thread message.
// ---------------------------------------------------------------------------
struct Error {
  cspt_status status;
  std::string message;
};

void set_last_error(std::string const& msg);
void clear_last_error();

#define CSPT_EXPECTS(cond, msg)                                               \
  do {                                                                        \
    if (!(cond)) throw ::cspt::Error{CSPT_INVALID_ARGUMENT, std::string(msg)}; \
  } while (0)

#define CSPT_CUDA_TRY(call)                                                          \
  do {                                                                               \
    cudaError_t const e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                         \
      (void)cudaGetLastError();                                                      \
      throw ::cspt::Error{e_ == cudaErrorMemoryAllocation ? CSPT_OUT_OF_MEMORY        \
                                                          : CSPT_CUDA_ERROR,          \
                          std::string("CUDA error at " __FILE__ ":") +               \
                            std::to_string(__LINE__) + ": " + cudaGetErrorString(e_)}; \
    }                                                                                \
  } while (0)

// Every kernel launch site is followed by CSPT_CHECK_LAUNCH(), which also
// counts the launch (cspt_launch_count()).  Launches recorded into a CUDA
// graph are taken back after the capture and counted per replay instead.
void count_launch();
void count_launches(uint64_t n);
void uncount_launches(uint64_t n);
#define CSPT_CHECK_LAUNCH()                     \
  do {                                          \
    ::cspt::count_launch();                     \
    CSPT_CUDA_TRY(cudaPeekAtLastError());       \
  } while (0)

// Optional event timing of named kernels on their launching stream
// (cspt_profile_*): a no-op unless profiling is enabled.
class KernelTimer {
 public:
  KernelTimer(char const* name, cudaStream_t stream);
  ~KernelTimer();
  KernelTimer(KernelTimer const&)            = delete;
  KernelTimer& operator=(KernelTimer const&) = delete;

 private:
  char const* name_;
  cudaStream_t stream_;
  cudaEvent_t start_ = nullptr;
  cudaEvent_t stop_  = nullptr;
};

// Runs `body`, turning exceptions into a status and the thread's message.
template <typename F>
cspt_status guarded(F&& body)
{
  try {
    clear_last_error();
    body();
    return CSPT_OK;
  } catch (Error const& e) {
    set_last_error(e.message);
    return e.status;
  } catch (std::exception const& e) {
    set_last_error(e.what());
    return CSPT_CUDA_ERROR;
  }
}

// ---------------------------------------------------------------------------
// memory: every device allocation goes through the caller's allocator, or,
// when none is given, the library's own stream-ordered pool on the current
// device.  The pool keeps what is freed for later calls (its release
// threshold is unbounded), where the device's default pool hands memory back
// to the CUDA driver at every synchronisation and maps it again on the next
// call.
// ---------------------------------------------------------------------------
cudaMemPool_t library_pool();

// A stream of the library on the current device (created on first use,
// non-blocking, kept for the life of the process), for work a long-lived
// object issues beside its caller's stream: memory ordered on it stays
// reusable across objects and threads, where a stream per object or per
// thread would leave the caching allocator's blocks on a dead stream.
cudaStream_t library_stream();

class Allocator {
 public:
  Allocator(cspt_allocator const* mr, cudaStream_t stream) : mr_(mr), stream_(stream) {}
  void* allocate(size_t bytes) const
  {
    if (bytes == 0) return nullptr;
    void* p = nullptr;
    if (mr_ && mr_->allocate) {
      p = mr_->allocate(mr_->ctx, bytes, stream_);
      if (!p) throw Error{CSPT_OUT_OF_MEMORY, "allocation of " + std::to_string(bytes) +
                                                 " bytes failed (caller allocator)"};
    } else {
      cudaError_t const e = cudaMallocFromPoolAsync(&p, bytes, library_pool(), stream_);
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw Error{CSPT_OUT_OF_MEMORY,
                    "allocation of " + std::to_string(bytes) + " bytes failed: " +
                      cudaGetErrorString(e)};
      }
    }
    return p;
  }
  void deallocate(void* p, size_t bytes) const
  {
    if (!p) return;
    if (mr_ && mr_->deallocate) {
      mr_->deallocate(mr_->ctx, p, bytes, stream_);
    } else {
      (void)cudaFreeAsync(p, stream_);
    }
  }
  cudaStream_t stream() const { return stream_; }
  cspt_allocator const* resource() const { return mr_; }

 private:
  cspt_allocator const* mr_;
  cudaStream_t stream_;
};

// Owning typed device buffer (freed on scope exit unless released).
template <typename T>
class Buffer {
 public:
  Buffer() = default;
  Buffer(Allocator const& a, size_t n) : a_(&a), n_(n)
  {
    p_ = static_cast<T*>(a.allocate(n * sizeof(T)));
  }
  Buffer(Buffer&& o) noexcept : a_(o.a_), p_(o.p_), n_(o.n_)
  {
    o.p_ = nullptr;
    o.n_ = 0;
  }
  Buffer& operator=(Buffer&& o) noexcept
  {
    reset();
    a_   = o.a_;
    p_   = o.p_;
    n_   = o.n_;
    o.p_ = nullptr;
    o.n_ = 0;
    return *this;
  }
  Buffer(Buffer const&)            = delete;
  Buffer& operator=(Buffer const&) = delete;
  ~Buffer() { reset(); }
  void reset()
  {
    if (p_ && a_) a_->deallocate(p_, n_ * sizeof(T));
    p_ = nullptr;
    n_ = 0;
  }
  T* release()
  {
    T* p = p_;
    p_   = nullptr;
    n_   = 0;
    return p;
  }
  T* data() const { return p_; }
  size_t size() const { return n_; }
  // takes ownership of n elements at p, allocated from a
  static Buffer adopt(Allocator const& a, T* p, size_t n)
  {
    Buffer b;
    b.a_ = &a;
    b.p_ = p;
    b.n_ = n;
    return b;
  }

 private:
  Allocator const* a_ = nullptr;
  T* p_               = nullptr;
  size_t n_           = 0;
};

// Reads one device value back to the host (synchronises the stream).
template <typename T>
T read_back(T const* dev, cudaStream_t stream)
{
  T h{};
  CSPT_CUDA_TRY(cudaMemcpyAsync(&h, dev, sizeof(T), cudaMemcpyDeviceToHost, stream));
  CSPT_CUDA_TRY(cudaStreamSynchronize(stream));
  return h;
}

inline unsigned grid_for(size_t n, unsigned block, unsigned cap = 1u << 20)
{
  size_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return static_cast<unsigned>(g);
}

// Streaming multiprocessors of the current device (cached per device).
int num_sms();
// Grid cap of `per_sm` blocks on every SM of the current device.
inline unsigned sm_grid(unsigned per_sm) { return static_cast<unsigned>(num_sms()) * per_sm; }

// Extra streams of the calling thread on the current device, for work that
// overlaps the caller's stream inside one call (created on first use;
// non-blocking with respect to the legacy default stream).  Stream 0 serves
// the copies and side kernels of a single call; stream 1 the polygon work a
// combined call runs beside a single call's streams.
constexpr int kSideStreams = 2;
cudaStream_t side_stream(int k = 0);

// Makes `waiter` wait for everything enqueued on `on` so far.
void stream_wait(cudaStream_t waiter, cudaStream_t on);

// Where a kernel reads the coordinates of the point at sorted position pos
// (a position in the quadtree's point_indices): through the permutation,
// x[point_indices[pos]] and y[point_indices[pos]] (the reference's gather,
// two dependent random reads), or from a copy of the points already in
// quadtree order, xy[2 pos] and xy[2 pos + 1] (one aligned vector read,
// coalesced across a warp).
template <typename T>
struct PointSource {
  uint32_t const* point_indices;
  T const* x;
  T const* y;
  T const* xy;  // interleaved (x, y) in quadtree order, or null

  __device__ __forceinline__ void load(uint64_t pos, T& px, T& py) const
  {
    if (xy) {
      if constexpr (sizeof(T) == 8) {
        double2 const v = reinterpret_cast<double2 const*>(xy)[pos];
        px              = v.x;
        py              = v.y;
      } else {
        float2 const v = reinterpret_cast<float2 const*>(xy)[pos];
        px             = v.x;
        py             = v.y;
      }
    } else {
      uint32_t const i = point_indices[pos];
      px               = x[i];
      py               = y[i];
    }
  }
};

// Caller's host arrays for result rows written to host memory.
struct HostRows {
  uint32_t* polygon_index;
  uint32_t* point_index;
  size_t capacity;  // rows each array holds
};

// Makes `main` wait for everything enqueued on `side` so far, at join() or
// when it goes out of scope (also while an exception unwinds), so that
// buffers released on `main` afterwards are no longer in use on `side`.
class StreamJoin {
 public:
  StreamJoin(cudaStream_t main, cudaStream_t side) : main_(main), side_(side) {}
  ~StreamJoin() { join(); }
  StreamJoin(StreamJoin const&)            = delete;
  StreamJoin& operator=(StreamJoin const&) = delete;
  void join();

 private:
  cudaStream_t main_;
  cudaStream_t side_;
};

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
template <typename T>
struct uint_of;
template <>
struct uint_of<float> {
  using type = uint32_t;
};
template <>
struct uint_of<double> {
  using type = uint64_t;
};

// cpp/include/cuspatial/detail/utility/floating_point.cuh:97-129: two values
// are equal when their biased integer images are at most 4 apart; NaN never
// equals anything.
template <typename T>
__host__ __device__ inline bool float_equal(T a, T b)
{
  using U = typename uint_of<T>::type;
  if (a != a || b != b) return false;
  U ua, ub;
  memcpy(&ua, &a, sizeof(T));
  memcpy(&ub, &b, sizeof(T));
  U const sign = U{1} << (8 * sizeof(U) - 1);
  U const ba   = (ua & sign) ? U(~ua + 1) : U(ua | sign);
  U const bb   = (ub & sign) ? U(~ub + 1) : U(ub | sign);
  return (ba >= bb ? ba - bb : bb - ba) <= 4u;
}

// Morton interleave (cpp/include/cuspatial/detail/utility/z_order.cuh:69-94),
// computed with shifts and masks.
__host__ __device__ inline uint32_t spread16(uint32_t v)
{
  v &= 0xFFFFu;
  v = (v | (v << 8)) & 0x00FF00FFu;
  v = (v | (v << 4)) & 0x0F0F0F0Fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}
__host__ __device__ inline uint32_t gather16(uint32_t v)
{
  v &= 0x55555555u;
  v = (v | (v >> 1)) & 0x33333333u;
  v = (v | (v >> 2)) & 0x0F0F0F0Fu;
  v = (v | (v >> 4)) & 0x00FF00FFu;
  v = (v | (v >> 8)) & 0x0000FFFFu;
  return v;
}

// v < lo || v > hi for bounds that are not NaN, on the integer pipe (GB300's
// float64 pipe runs comparisons at a small fraction of the integer rate).
// Non-NaN doubles order as their sign-magnitude bits read as a signed
// integer after negating the negative ones (both zeros map to 0); a NaN v
// compares false, as the float64 comparisons do.
__device__ inline long long ordered_bits(double v)
{
  long long const b = __double_as_longlong(v);
  long long const m = b & 0x7FFFFFFFFFFFFFFFll;
  return b < 0 ? -m : m;
}
__device__ inline bool outside_closed(double v, double lo, double hi)
{
  long long const m = __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFll;
  if (m > 0x7FF0000000000000ll) return false;  // NaN
  long long const k = ordered_bits(v);
  return k < ordered_bits(lo) || k > ordered_bits(hi);
}
__device__ inline bool outside_closed(float v, float lo, float hi) { return v < lo || v > hi; }

// static_cast<uint16_t>(t / s) for t >= 0 (the reference's cell index,
// phase_1.cuh:73-85) without a float64 division in the common case.  With
// r = fl(1/s) (host-rounded) and q0 = fl(t * r):
//   |q0 - t/s| <= (t/s)(2^-52 + 2^-106)   and   |fl(t/s) - t/s| <= 2^-53 t/s,
// so for t/s < 2^16 the two differ by less than 2^-35.  When q0 lies more
// than 2^-30 away from every integer, q0 and fl(t/s) have the same integer
// part; the fraction test reads q0's bits.  Every other case (near an
// integer, below 2^-30, 2^16 and above, non-finite) divides.
__device__ inline uint16_t cell_of_quotient(double t, double s, double r)
{
  double const q0          = t * r;
  unsigned long long const b = static_cast<unsigned long long>(__double_as_longlong(q0));
  int const e              = static_cast<int>((b >> 52) & 0x7FFull) - 1023;
  if (e >= 0 && e < 16 && !(b >> 63)) {
    unsigned long long const m    = (b & ((1ull << 52) - 1ull)) | (1ull << 52);
    int const sh                  = 52 - e;  // fraction bits, >= 37
    unsigned long long const frac = m & ((1ull << sh) - 1ull);
    unsigned long long const mg   = 1ull << (sh - 30);
    if (frac > mg && frac < (1ull << sh) - mg) return static_cast<uint16_t>(m >> sh);
  } else if (b > 0x3E10000000000000ull && b < 0x3FEFFFFFFF800000ull) {
    return 0;  // 2^-30 < q0 < 1 - 2^-30 (positive doubles order as integers)
  }
  return static_cast<uint16_t>(t / s);
}
__device__ inline uint16_t cell_of_quotient(float t, float s, float)
{
  return static_cast<uint16_t>(t / s);
}

// Explicitly rounded arithmetic: the library is compiled with -fmad=false,
// and the few products the reference's build contracts into FMAs are written
// as fma_rn.
__device__ inline double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ inline float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }

template <typename T>
__device__ inline T ldg(T const* p)
{
  return __ldg(p);
}

}  // namespace cspt
