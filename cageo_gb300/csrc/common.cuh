// common.cuh -- shared device/host helpers for the cageo kernels.
#pragma once
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>
#include "cageo.h"

namespace cageo {

// ---- error reporting (thread-local last error; see cageo_last_error_string)
void set_error(const char* fmt, ...);
cageo_status cuda_fail(cudaError_t e, const char* what);

#define CAGEO_CUDA(call)                                        \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) return ::cageo::cuda_fail(e_, #call); \
  } while (0)

#define CAGEO_CHECK_ARG(cond, msg)                      \
  do {                                                  \
    if (!(cond)) {                                      \
      ::cageo::set_error("invalid argument: %s", msg);  \
      return CAGEO_ERR_ARGUMENT;                        \
    }                                                   \
  } while (0)

// Grids larger than this are refused (int32 cell indices in the kernels).
constexpr int64_t kMaxCells = (int64_t)1 << 31;

inline bool valid_dims(int W, int H) {
  return W > 0 && H > 0 && (int64_t)W * H < kMaxCells;
}

// Stream-ordered scratch: the caller's workspace when given, else
// cudaMallocAsync / cudaFreeAsync on the stream.
struct Scratch {
  void* ptr = nullptr;
  bool owned = false;
  cudaStream_t stream = 0;
  cageo_status acquire(void* given, size_t given_bytes, size_t need,
                       cudaStream_t s);
  ~Scratch();
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// ---- per-device launch set-up ----------------------------------------------
// A kernel's launch set-up (its dynamic shared-memory limit raised, the
// number of blocks a cooperative launch may have) is made once per device
// and kept in a process-wide table.  Function attributes belong to the
// device, so each device is set up on its own.  Host threads may race to
// fill an entry: each runs the (idempotent) set-up and stores the same value.
constexpr int kMaxDevices = 64;
struct PerDevice {
  std::atomic<int> value[kMaxDevices];  // 0 until set up (static storage starts zeroed)
};

// *out = the cached value for the current device; `setup(dev, &v)` makes
// it (v >= 1) the first time.
template <typename SetUp>
cageo_status per_device(PerDevice& cache, int* out, SetUp&& setup) {
  int dev = 0;
  CAGEO_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("device %d is beyond the %d devices a process may use", dev, kMaxDevices);
    return CAGEO_ERR_ARGUMENT;
  }
  int v = cache.value[dev].load(std::memory_order_acquire);
  if (v == 0) {
    cageo_status st = setup(dev, &v);
    if (st) return st;
    cache.value[dev].store(v, std::memory_order_release);
  }
  *out = v;
  return CAGEO_OK;
}

// Blocks of `fn` (`threads` threads, `smem` bytes of dynamic shared memory)
// that device `dev` holds at once: the largest grid of a cooperative launch.
inline cageo_status resident_blocks(const void* fn, int threads, size_t smem, int dev,
                                    int* out) {
  int sms = 0, per = 0;
  CAGEO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CAGEO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, threads, smem));
  *out = (per > 1 ? per : 1) * (sms > 1 ? sms : 1);
  return CAGEO_OK;
}

// ---- device helpers --------------------------------------------------------
constexpr float kInf = __builtin_huge_valf();

// Monotone map float -> uint32 so that unsigned order equals float order
// (for non-NaN values); used for atomicMin/atomicMax on floats.
__host__ __device__ inline uint32_t float_to_ordered(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float ordered_to_float(uint32_t u) {
  uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  float f;
  memcpy(&f, &v, 4);
  return f;
}

// Appends for every lane of the calling warp whose `pred` is true, with a
// single atomicAdd per warp; returns the lane's slot, or 0xffffffff when
// `pred` is false.  All active lanes of the warp must call it together.
__device__ __forceinline__ unsigned int warp_append(unsigned int* counter, bool pred) {
  const unsigned int active = __activemask();
  const unsigned int ball = __ballot_sync(active, pred);
  if (!ball) return 0xffffffffu;
  unsigned int lane;
  asm volatile("mov.u32 %0, %%laneid;" : "=r"(lane));
  const int leader = __ffs(ball) - 1;
  unsigned int base = 0;
  if ((int)lane == leader) base = atomicAdd(counter, (unsigned int)__popc(ball));
  base = __shfl_sync(active, base, leader);
  return pred ? base + (unsigned int)__popc(ball & ((1u << lane) - 1u)) : 0xffffffffu;
}

// Grid-wide barrier for persistent kernels launched cooperatively (all
// blocks co-resident).  One thread per block arrives on `count`; the last
// arrival resets it and bumps `generation`, which the others poll with an
// exponential back-off.  `count` and `generation` live on different
// 128-byte lines so arrivals do not queue behind polls.  Every wait is
// bounded: after the poll limit the block records an error in *err and
// returns false; callers then leave their loops.
struct GridSync {
  unsigned int* count;
  unsigned int* generation;
  int* err;
};

// Scalar-block slots used by GridSync (uint32 indices: separate lines).
constexpr int kBarCountSlot = 32;
constexpr int kBarGenSlot = 64;
constexpr int kScalarSlots = 96;

// Asynchronous 4-byte global -> shared copy (LDGSTS): many can be in flight
// per thread without holding registers.  Complete them with cp_async_wait().
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned int sa = (unsigned int)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

__device__ inline bool grid_barrier(const GridSync& g, unsigned int nblocks) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = g.generation;
    unsigned int my = *gen;
    __threadfence();
    unsigned int arrived = atomicAdd(g.count, 1u);
    ok = 1;
    if (arrived == nblocks - 1) {
      *(volatile unsigned int*)g.count = 0u;
      __threadfence();
      atomicAdd(g.generation, 1u);
    } else {
      unsigned int ns = 32;
      long long polls = 0;
      while (*gen == my) {
        if (++polls > 20000000LL) {  // several seconds
          atomicExch(g.err, 1);
          ok = 0;
          break;
        }
        if ((polls & 63) == 0 && *((volatile int*)g.err)) { ok = 0; break; }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

}  // namespace cageo
