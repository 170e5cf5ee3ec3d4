// fl_device.cuh -- device-side helpers shared by the library's kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "fl_internal.cuh"

namespace fl {

// Kernel launch accounting: block (0,0,0) thread 0 of every kernel of this
// library bumps a device counter of its translation unit; the per-unit
// counters are summed by fl_kernel_launch_count().
static __device__ unsigned long long g_launch_counter;

__device__ __forceinline__ void note_launch() {
  if ((blockIdx.x | blockIdx.y | blockIdx.z | threadIdx.x | threadIdx.y) == 0)
    atomicAdd(&g_launch_counter, 1ull);
}

__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(int* p, int v) {
  asm volatile("st.relaxed.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The records of a warp's 32 elements are staged in shared memory for a
// coalesced copy-out, lane l's record at stage + l (NREC + 1): with the one
// float4 of padding, the eight lanes of one shared-memory wavefront (16-B
// stores) write eight different bank groups (records 128 or 192 B apart
// would put them all in one or two).  stage_pos maps a position of the
// warp's contiguous record run (position 32 k + lane, k unrolled) to its
// padded place, idx + idx / NREC, written so that a lane keeps one or three
// offset registers and k enters as an immediate: 36 k + lane + lane / 8 for
// 8-float4 records; for 12- (6-) float4 records every 3 k cover 8 (16)
// records, 104 (112) padded float4.  The P2 pass stages 6-float4 row slices
// the same way (lanes 96 B apart would share two bank groups per four), the
// pressure-stabilisation pass its 8-float4 records.
template <int NREC>
__device__ __forceinline__ int stage_pos(int k, int lane) {
  static_assert(NREC == 6 || NREC == 8 || NREC == 12, "staged records are 6, 8 or 12 float4");
  if (NREC == 8) return 36 * k + lane + (lane >> 3);
  const int r = 32 * (k % 3) + lane;
  return 96 / NREC * (NREC + 1) * (k / 3) + r + (int)((unsigned)r / (unsigned)NREC);
}

// 32 bytes from a 32-byte aligned global address that no thread writes
// during the kernel, in one 256-bit load (ld.global.nc.v8, sm_100 and later).
__device__ __forceinline__ void ldg256(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

// First error wins; `where` records the element / row that raised it.
__device__ __forceinline__ void set_err(ErrWord* err, int code, int where) {
  if (atomicCAS(&err->code, 0, code) == 0) err->where = where;
}

// Bisection in a sorted CSR row [b, e) (csr_sparsity_pos,
// femtools/Sparse_Tools.F90:2411-2517); -1 when j is not in the row.
__device__ __forceinline__ int csr_find(const int32_t* __restrict__ colm, int b, int e, int j) {
  int lo = b, hi = e - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    int c = __ldg(colm + mid);
    if (c == j) return mid;
    if (c < j) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

template <int THREADS>
__device__ __forceinline__ int64_t block_sum_i64(int64_t v, int64_t* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < THREADS / 32 ? red[lane] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  return v;  // valid in thread 0
}

static __global__ void k_copy_i64_to_i32(const int64_t* __restrict__ in, int32_t* __restrict__ out,
                                         int64_t n) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = (int32_t)in[k];
}

static __global__ void k_fill_i32(int32_t* __restrict__ p, int64_t n, int32_t v) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    p[k] = v;
}

// Host reader of this translation unit's launch counter.
static inline unsigned long long unit_launches() {
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_launch_counter, sizeof(v)) != cudaSuccess) return 0;
  return v;
}

// Reads and clears the error word; non-OK status carries `what` + detail.
int check_err(ErrWord* d_err, cudaStream_t s, const char* what);

}  // namespace fl
