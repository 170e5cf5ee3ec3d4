// fl_gnn.cu -- learned warm start for the pressure solve: a message-passing
// network over the mesh graph, trained on the GPU by the kernels below.
//
// The network predicts the next pressure of a sequence of Poisson solves from
// node features (previous two pressures, right-hand side, coordinates):
//
//   f_i  = [p1_i/s, p2_i/s, b_i/sb, 2x_i-1, 2y_i-1, 2z_i-1, 0 x 10]   (16)
//   h0_i = relu(We f_i + be)                                            (64)
//   for l = 1..3:  a_i = mean_{j in N(i), j != i} h_j                   (64)
//                  h_i <- h_i + relu(Wl [h_i ; a_i] + bl)                (64)
//   p_i  = 2 p1_i - p2_i + s (wd . h_i + bd)
//
// with s = max|p1| and sb = max|b|; N(i) is the node's row of the mesh's
// first-order sparsity pattern (the same graph the matrix lives on).  Weights
// and activations are BF16, every product is accumulated in FP32 on the
// tensor cores (mma.sync m16n8k16 bf16 -> f32), and the FP32 master weights
// are updated by Adam.  The loss is the mean squared normalised error over
// the active (non-Dirichlet) nodes.  Weight gradients are summed over node
// tiles by a fixed set of blocks and then over blocks in a fixed order, so
// training is deterministic.
//
// The reference has no counterpart: this is the learned-initial-guess
// extension of the petsc_solve call on the pressure system; the solver still
// runs to the same tolerance from the predicted guess.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "fl_internal.cuh"
#include "fl_device.cuh"

namespace fl {

unsigned long long launches_gnn() { return unit_launches(); }

namespace {

constexpr int kW = 64;        // width
constexpr int kF = 16;        // input features (6 used), one mma K step
constexpr int kLayers = 3;
constexpr int kTM = 64;       // nodes per tile
constexpr int kTh = 128;      // threads of the tile kernels (4 warps x 16 nodes)
constexpr int kPersist = 456; // blocks (3 per SM) of the reduction-over-nodes kernels

// flat FP32 parameter vector
constexpr int kOffWe = 0;                    // [64][16]
constexpr int kOffBe = kOffWe + kW * kF;     // [64]
constexpr int kOffL = kOffBe + kW;           // per layer: W [64][128], b [64]
constexpr int kLayerSize = kW * 2 * kW + kW;
constexpr int kOffWd = kOffL + kLayers * kLayerSize;  // [64]
constexpr int kOffBd = kOffWd + kW;                   // [1]
constexpr int kParams = kOffBd + 1;
constexpr int kPartStride = kW * 2 * kW + kW;  // largest per-block partial (a layer)

// padded shared-memory row lengths (bf16): conflict-free fragment loads
constexpr int kLd16 = kF + 8;
constexpr int kLd64 = kW + 8;
constexpr int kLd128 = 2 * kW + 8;

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t ld32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// D += A B for one m16n8k16 tile (A row-major 16x16, B column-major 16x8).
__device__ __forceinline__ void mma_bf16(float* d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// acc[NT][4] += X[16 rows][K] * B, where B[k][n] = Bs[n][k] (Bs row-major,
// k contiguous; NT tiles of 8 columns).  X rows have stride LDX, Bs rows LDB.
template <int K, int NT, int LDX, int LDB>
__device__ __forceinline__ void warp_gemm(const bf16* X, const bf16* Bs, float (*acc)[4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int ks = 0; ks < K / 16; ++ks) {
    const int k0 = ks * 16 + t * 2;
    const uint32_t a0 = ld32(X + g * LDX + k0), a1 = ld32(X + (g + 8) * LDX + k0);
    const uint32_t a2 = ld32(X + g * LDX + k0 + 8), a3 = ld32(X + (g + 8) * LDX + k0 + 8);
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
      const bf16* b = Bs + (nt * 8 + g) * LDB + k0;
      mma_bf16(acc[nt], a0, a1, a2, a3, ld32(b), ld32(b + 8));
    }
  }
}

struct Inputs {
  int n;
  const double* p1;
  const double* p2;
  const double* b;
  const double* X;        // (n, 3)
  const float* scal;      // [0] = s, [1] = sb
};

__device__ __forceinline__ float scale_of(float v) { return v > 0.0f ? v : 1.0f; }

// Features in FP32: the pressures and rhs rounded to float, times the float
// reciprocal of their scale (no FP64 divide).
__device__ __forceinline__ void features(const Inputs& in, int i, float* f) {
  const float is = 1.0f / scale_of(in.scal[0]), isb = 1.0f / scale_of(in.scal[1]);
  f[0] = __double2float_rn(in.p1[i]) * is;
  f[1] = __double2float_rn(in.p2[i]) * is;
  f[2] = __double2float_rn(in.b[i]) * isb;
  f[3] = (float)(2.0 * in.X[3 * i] - 1.0);
  f[4] = (float)(2.0 * in.X[3 * i + 1] - 1.0);
  f[5] = (float)(2.0 * in.X[3 * i + 2] - 1.0);
#pragma unroll
  for (int k = 6; k < kF; ++k) f[k] = 0.0f;
}

// order-independent max of |p1| and |b| (atomicMax on the bits of
// non-negative floats)
__global__ void k_gnn_scales(int n, const double* __restrict__ p1, const double* __restrict__ b, float* scal) {
  note_launch();
  float a = 0.0f, c = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    a = fmaxf(a, (float)fabs(p1[i]));
    c = fmaxf(c, (float)fabs(b[i]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
    c = fmaxf(c, __shfl_xor_sync(0xffffffffu, c, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(reinterpret_cast<unsigned*>(scal), __float_as_uint(a));
    atomicMax(reinterpret_cast<unsigned*>(scal + 1), __float_as_uint(c));
  }
}

__global__ void k_gnn_inv_deg(int n, const int32_t* __restrict__ findrm, float* __restrict__ inv) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int d = findrm[i + 1] - findrm[i] - 1;  // the diagonal is not a neighbour
    inv[i] = d > 0 ? 1.0f / (float)d : 0.0f;
  }
}

// h0 = relu(We f + be); Z0 = We f + be (bf16, stored when Z is not null)
__global__ void __launch_bounds__(kTh) k_gnn_encode(Inputs in, const bf16* __restrict__ We,
                                                    const float* __restrict__ be, bf16* __restrict__ Z,
                                                    bf16* __restrict__ H) {
  note_launch();
  __shared__ __align__(16) bf16 Fs[kTM * kLd16];
  __shared__ __align__(16) bf16 Ws[kW * kLd16];
  for (int k = threadIdx.x; k < kW * kF; k += kTh) Ws[(k / kF) * kLd16 + k % kF] = We[k];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int ntiles = (in.n + kTM - 1) / kTM;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int base = tile * kTM;
    __syncthreads();
    if (threadIdx.x < kTM) {
      const int i = base + threadIdx.x;
      float f[kF];
      if (i < in.n) features(in, i, f);
      else
        for (int k = 0; k < kF; ++k) f[k] = 0.0f;
      for (int k = 0; k < kF; ++k) Fs[threadIdx.x * kLd16 + k] = __float2bfloat16_rn(f[k]);
    }
    __syncthreads();
    float acc[8][4] = {};
    warp_gemm<kF, 8, kLd16, kLd16>(Fs + w * 16 * kLd16, Ws, acc);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = base + w * 16 + g + 8 * h, c = nt * 8 + t * 2;
        if (row >= in.n) continue;
        const float z0 = acc[nt][2 * h] + be[c], z1 = acc[nt][2 * h + 1] + be[c + 1];
        if (Z) *reinterpret_cast<__nv_bfloat162*>(Z + (int64_t)row * kW + c) = __floats2bfloat162_rn(z0, z1);
        *reinterpret_cast<__nv_bfloat162*>(H + (int64_t)row * kW + c) =
            __floats2bfloat162_rn(fmaxf(z0, 0.0f), fmaxf(z1, 0.0f));
      }
  }
}

// One message-passing layer on a tile of 64 nodes: the tile's own states h
// and the means a of their neighbours' states (gathered by the four warps,
// one node at a time, FP32 sums of the bf16 rows in pattern order) are
// staged in shared memory as [h | a], then on the tensor cores
// z = Wl [h ; a] + bl and h' = h + relu(z).  A and Z (the values the
// backward pass needs) are stored only when their pointers are not null.
__global__ void __launch_bounds__(kTh) k_gnn_layer_fwd(int n, const int32_t* __restrict__ findrm,
                                                       const int32_t* __restrict__ colm,
                                                       const float* __restrict__ inv_deg,
                                                       const bf16* __restrict__ Hin, const bf16* __restrict__ Wl,
                                                       const float* __restrict__ bl, bf16* __restrict__ A,
                                                       bf16* __restrict__ Z, bf16* __restrict__ Hout) {
  note_launch();
  __shared__ __align__(16) bf16 Xs[kTM * kLd128];
  __shared__ __align__(16) bf16 Ws[kW * kLd128];
  for (int k = threadIdx.x; k < kW * 16; k += kTh) {
    const int r = k >> 4, q = k & 15;
    *reinterpret_cast<uint4*>(Ws + r * kLd128 + q * 8) = *reinterpret_cast<const uint4*>(Wl + r * 2 * kW + q * 8);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int ntiles = (n + kTM - 1) / kTM;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int base = tile * kTM;
    __syncthreads();
    for (int k = threadIdx.x; k < kTM * 8; k += kTh) {
      const int r = k >> 3, q = k & 7, i = base + r;
      uint4 v = {0u, 0u, 0u, 0u};
      if (i < n) v = *reinterpret_cast<const uint4*>(Hin + (int64_t)i * kW + q * 8);
      *reinterpret_cast<uint4*>(Xs + r * kLd128 + q * 8) = v;
    }
    {
      // four nodes per warp at a time, eight lanes per node, eight features
      // (one 16-byte load) per lane.  The eight lanes of a node first load
      // eight of its column indices, then every row load of those eight
      // neighbours is issued before the sums (pattern order is kept).
      const int sub = lane >> 3, q = lane & 7;
      for (int r = w * 4 + sub; r < kTM; r += kTh / 8) {
        const int i = base + r;
        float s[8] = {};
        const int b = i < n ? findrm[i] : 0, e = i < n ? findrm[i + 1] : 0;
        const int len = __reduce_max_sync(0xffffffffu, e - b);  // longest row of the warp's nodes
        for (int k0 = 0; k0 < len; k0 += 8) {
          const int kk = b + k0 + q;
          const int jl = kk < e ? colm[kk] : -1;
          uint4 v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int j = __shfl_sync(0xffffffffu, jl, u, 8);
            v[u] = (j >= 0 && j != i) ? *reinterpret_cast<const uint4*>(Hin + (int64_t)j * kW + q * 8)
                                      : make_uint4(0u, 0u, 0u, 0u);
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int j = __shfl_sync(0xffffffffu, jl, u, 8);
            if (j < 0 || j == i) continue;
            const __nv_bfloat162* h2 = reinterpret_cast<const __nv_bfloat162*>(&v[u]);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const float2 h = __bfloat1622float2(h2[c]);
              s[2 * c] += h.x;
              s[2 * c + 1] += h.y;
            }
          }
        }
        if (i < n) {
          const float d = inv_deg[i];
#pragma unroll
          for (int u = 0; u < 8; ++u) s[u] *= d;
        }
        uint4 out;
        __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(&out);
#pragma unroll
        for (int u = 0; u < 4; ++u) o2[u] = __floats2bfloat162_rn(s[2 * u], s[2 * u + 1]);
        *reinterpret_cast<uint4*>(Xs + r * kLd128 + kW + q * 8) = out;
        if (A && i < n) *reinterpret_cast<uint4*>(A + (int64_t)i * kW + q * 8) = out;
      }
    }
    __syncthreads();
    float acc[8][4] = {};
    warp_gemm<2 * kW, 8, kLd128, kLd128>(Xs + w * 16 * kLd128, Ws, acc);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = w * 16 + g + 8 * h, row = base + r, c = nt * 8 + t * 2;
        if (row >= n) continue;
        const float z0 = acc[nt][2 * h] + bl[c], z1 = acc[nt][2 * h + 1] + bl[c + 1];
        const float2 hin = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(Xs + r * kLd128 + c));
        if (Z) *reinterpret_cast<__nv_bfloat162*>(Z + (int64_t)row * kW + c) = __floats2bfloat162_rn(z0, z1);
        *reinterpret_cast<__nv_bfloat162*>(Hout + (int64_t)row * kW + c) =
            __floats2bfloat162_rn(hin.x + fmaxf(z0, 0.0f), hin.y + fmaxf(z1, 0.0f));
      }
  }
}

struct DecodeArgs {
  Inputs in;
  const bf16* H;        // h3
  const bf16* wd;       // bf16 decoder weights
  const float* bd;      // fp32 bias (master)
  double* pred;         // may be null
  const double* target; // null: inference only
  const uint8_t* mask;  // active nodes (may be null: all)
  float inv_nact;       // 1 / number of active nodes
  float* dH;            // [n][64] gradient w.r.t. h3 (training)
  float* part;          // [gridDim][66]: dwd, dbd, loss
  int energy;           // loss in the energy norm of the matrix
  double* e;            // energy loss: normalised error (first pass writes it)
  const double* Ke;     // energy loss: K e (second pass reads it)
};

// o = wd . h3 + bd; prediction; training: e, dL/do, dh3, decoder partials.
// Loss in the energy norm (e^T K e over the active nodes) takes two passes:
// the first writes e (Ke is null), the second, after K e, the gradients.
__global__ void __launch_bounds__(kTh) k_gnn_decode(DecodeArgs D) {
  note_launch();
  __shared__ float red[kTh / 32][kW + 2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const float2 wd = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(D.wd)[lane]);
  const float bd = D.bd[0];
  const double s = scale_of(D.in.scal[0]);
  float2 gw = {0.0f, 0.0f};
  float gb = 0.0f, loss = 0.0f;
  const int nw = gridDim.x * (kTh >> 5);
  for (int i = blockIdx.x * (kTh >> 5) + w; i < D.in.n; i += nw) {
    const float2 h = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(D.H + (int64_t)i * kW)[lane]);
    float o = wd.x * h.x + wd.y * h.y;
#pragma unroll
    for (int k = 16; k > 0; k >>= 1) o += __shfl_xor_sync(0xffffffffu, o, k);
    o += bd;
    const double ext = 2.0 * D.in.p1[i] - D.in.p2[i];
    if (D.pred && lane == 0) D.pred[i] = ext + s * (double)o;
    if (D.target) {
      const bool act = !D.mask || D.mask[i];
      float go;
      if (D.energy && !D.Ke) {
        if (lane == 0) D.e[i] = act ? (ext - D.target[i]) / s + (double)o : 0.0;
        continue;
      } else if (D.energy) {
        const double ke = act ? D.Ke[i] : 0.0;
        go = (float)(2.0 * ke) * D.inv_nact;
        loss += lane == 0 ? (float)(D.e[i] * ke) : 0.0f;
      } else {
        const float e = act ? (float)((ext - D.target[i]) / s) + o : 0.0f;
        go = 2.0f * e * D.inv_nact;
        loss += lane == 0 ? e * e : 0.0f;
      }
      gb += lane == 0 ? go : 0.0f;
      gw.x += go * h.x;
      gw.y += go * h.y;
      reinterpret_cast<float2*>(D.dH + (int64_t)i * kW)[lane] = make_float2(go * wd.x, go * wd.y);
    }
  }
  if (!D.target || (D.energy && !D.Ke)) return;
  red[w][2 * lane] = gw.x;
  red[w][2 * lane + 1] = gw.y;
  if (lane == 0) {
    red[w][kW] = gb;
    red[w][kW + 1] = loss;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kW + 2; k += kTh) {
    float v = 0.0f;
    for (int q = 0; q < kTh / 32; ++q) v += red[q][k];
    D.part[(int64_t)blockIdx.x * (kW + 2) + k] = v;
  }
}

// Layer backward, input gradients: dZ = dH' * (Z > 0) (bf16);
// [dh ; da] = Wl^T dZ;  dHin = dH' + dh (residual);  dA = da.
__global__ void __launch_bounds__(kTh) k_gnn_bwd_dx(int n, const float* __restrict__ dHn,
                                                    const bf16* __restrict__ Z, const bf16* __restrict__ Wl,
                                                    float* __restrict__ dHin, float* __restrict__ dA) {
  note_launch();
  __shared__ __align__(16) bf16 dZs[kTM * kLd64];
  __shared__ __align__(16) bf16 Wt[2 * kW * kLd64];  // Wt[in][out]
  for (int k = threadIdx.x; k < kW * 2 * kW; k += kTh) {
    const int o = k / (2 * kW), c = k % (2 * kW);
    Wt[c * kLd64 + o] = Wl[k];
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int ntiles = (n + kTM - 1) / kTM;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int base = tile * kTM;
    __syncthreads();
    for (int k = threadIdx.x; k < kTM * (kW / 2); k += kTh) {
      const int r = k / (kW / 2), c = 2 * (k % (kW / 2)), i = base + r;
      float2 d = {0.0f, 0.0f};
      if (i < n) {
        const float2 gz = *reinterpret_cast<const float2*>(dHn + (int64_t)i * kW + c);
        const float2 z = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(Z + (int64_t)i * kW + c));
        d.x = z.x > 0.0f ? gz.x : 0.0f;
        d.y = z.y > 0.0f ? gz.y : 0.0f;
      }
      *reinterpret_cast<__nv_bfloat162*>(dZs + r * kLd64 + c) = __floats2bfloat162_rn(d.x, d.y);
    }
    __syncthreads();
    float acc[16][4] = {};
    warp_gemm<kW, 16, kLd64, kLd64>(dZs + w * 16 * kLd64, Wt, acc);
#pragma unroll
    for (int nt = 0; nt < 16; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = base + w * 16 + g + 8 * h, c = nt * 8 + t * 2;
        if (row >= n) continue;
        if (c < kW) {
          const float2 gz = *reinterpret_cast<const float2*>(dHn + (int64_t)row * kW + c);
          *reinterpret_cast<float2*>(dHin + (int64_t)row * kW + c) =
              make_float2(gz.x + acc[nt][2 * h], gz.y + acc[nt][2 * h + 1]);
        } else {
          *reinterpret_cast<float2*>(dA + (int64_t)row * kW + c - kW) =
              make_float2(acc[nt][2 * h], acc[nt][2 * h + 1]);
        }
      }
  }
}

// Layer backward, weight gradients: dWl = dZ^T [h ; a], dbl = sum dZ, summed
// over the node tiles of this block; one partial per block.  Eight warps:
// warp w owns output rows 16 (w % 4) .. +16 and input columns 64 (w / 4) ..
// +64.  Tiles are loaded eight channels (16 bytes of bf16, 32 of fp32) at a
// time and transposed into shared memory ([channel][node]).
constexpr int kThW = 256;
__global__ void __launch_bounds__(kThW) k_gnn_bwd_dw(int n, const float* __restrict__ dHn,
                                                     const bf16* __restrict__ Z, const bf16* __restrict__ Hin,
                                                     const bf16* __restrict__ A, float* __restrict__ part) {
  note_launch();
  __shared__ __align__(16) bf16 dZt[kW * kLd64];      // [out][node]
  __shared__ __align__(16) bf16 Xt[2 * kW * kLd64];   // [in][node]
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int wm = w & 3, wn = w >> 2;
  float acc[8][4] = {};
  float db = 0.0f;  // thread c < 64: bias gradient of output channel c
  const int ntiles = (n + kTM - 1) / kTM;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int base = tile * kTM;
    __syncthreads();
    for (int k = threadIdx.x; k < kTM * (kW / 8); k += kThW) {
      const int r = k >> 3, c0 = (k & 7) * 8, i = base + r;
      float d[8] = {};
      uint4 hv = {0u, 0u, 0u, 0u}, av = hv;
      if (i < n) {
        const uint4 zv = *reinterpret_cast<const uint4*>(Z + (int64_t)i * kW + c0);
        const float4 g0 = *reinterpret_cast<const float4*>(dHn + (int64_t)i * kW + c0);
        const float4 g1 = *reinterpret_cast<const float4*>(dHn + (int64_t)i * kW + c0 + 4);
        hv = *reinterpret_cast<const uint4*>(Hin + (int64_t)i * kW + c0);
        av = *reinterpret_cast<const uint4*>(A + (int64_t)i * kW + c0);
        const bf16* z8 = reinterpret_cast<const bf16*>(&zv);
        const float gg[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
#pragma unroll
        for (int u = 0; u < 8; ++u) d[u] = __bfloat162float(z8[u]) > 0.0f ? gg[u] : 0.0f;
      }
      const bf16* h8 = reinterpret_cast<const bf16*>(&hv);
      const bf16* a8 = reinterpret_cast<const bf16*>(&av);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        dZt[(c0 + u) * kLd64 + r] = __float2bfloat16_rn(d[u]);
        Xt[(c0 + u) * kLd64 + r] = h8[u];
        Xt[(kW + c0 + u) * kLd64 + r] = a8[u];
      }
    }
    __syncthreads();
    warp_gemm<kTM, 8, kLd64, kLd64>(dZt + wm * 16 * kLd64, Xt + wn * kW * kLd64, acc);
    if (threadIdx.x < kW)
      for (int r = 0; r < kTM; ++r) db += __bfloat162float(dZt[threadIdx.x * kLd64 + r]);
  }
  float* out = part + (int64_t)blockIdx.x * kPartStride;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int o = wm * 16 + g + 8 * h, c = wn * kW + nt * 8 + t * 2;
      out[o * 2 * kW + c] = acc[nt][2 * h];
      out[o * 2 * kW + c + 1] = acc[nt][2 * h + 1];
    }
  if (threadIdx.x < kW) out[kW * 2 * kW + threadIdx.x] = db;
}

// Aggregation backward: dHin_j += sum_{i in row j, i != j} inv_deg_i dA_i
// (the pattern is symmetric).
__global__ void k_gnn_agg_bwd(int n, const int32_t* __restrict__ findrm, const int32_t* __restrict__ colm,
                              const float* __restrict__ inv_deg, const float* __restrict__ dA,
                              float* __restrict__ dHin) {
  note_launch();
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < n; j += nw) {
    float2 s = {0.0f, 0.0f};
    const int b = findrm[j], e = findrm[j + 1];
    // the lanes load 32 column indices (and their inverse degrees) at a time,
    // then the rows of up to eight neighbours are loaded before they are summed
    for (int k0 = b; k0 < e; k0 += 32) {
      const int il = k0 + lane < e ? colm[k0 + lane] : -1;
      const float dl = il >= 0 ? inv_deg[il] : 0.0f;
      const int cnt = min(32, e - k0);
      for (int u0 = 0; u0 < cnt; u0 += 8) {
        float2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = __shfl_sync(0xffffffffu, il, (u0 + u) & 31);
          v[u] = (u0 + u < cnt && i != j) ? reinterpret_cast<const float2*>(dA + (int64_t)i * kW)[lane]
                                           : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = __shfl_sync(0xffffffffu, il, (u0 + u) & 31);
          const float d = __shfl_sync(0xffffffffu, dl, (u0 + u) & 31);
          if (u0 + u >= cnt || i == j) continue;
          s.x = fmaf(d, v[u].x, s.x);
          s.y = fmaf(d, v[u].y, s.y);
        }
      }
    }
    float2* o = reinterpret_cast<float2*>(dHin + (int64_t)j * kW) + lane;
    const float2 c = *o;
    *o = make_float2(c.x + s.x, c.y + s.y);
  }
}

// Encoder backward: dZ0 = dH0 * (Z0 > 0); dWe = dZ0^T F; dbe = sum dZ0.
__global__ void __launch_bounds__(kTh) k_gnn_bwd_enc(Inputs in, const float* __restrict__ dH0,
                                                     const bf16* __restrict__ Z0, float* __restrict__ part) {
  note_launch();
  __shared__ __align__(16) bf16 dZt[kW * kLd64];  // [out][node]
  __shared__ __align__(16) bf16 Ft[kF * kLd64];   // [feature][node]
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float acc[2][4] = {};
  float db = 0.0f;
  const int ntiles = (in.n + kTM - 1) / kTM;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int base = tile * kTM;
    __syncthreads();
    for (int k = threadIdx.x; k < kTM * (kW / 8); k += kTh) {
      const int r = k >> 3, c0 = (k & 7) * 8, i = base + r;
      float d[8] = {};
      if (i < in.n) {
        const uint4 zv = *reinterpret_cast<const uint4*>(Z0 + (int64_t)i * kW + c0);
        const float4 g0 = *reinterpret_cast<const float4*>(dH0 + (int64_t)i * kW + c0);
        const float4 g1 = *reinterpret_cast<const float4*>(dH0 + (int64_t)i * kW + c0 + 4);
        const bf16* z8 = reinterpret_cast<const bf16*>(&zv);
        const float gg[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
#pragma unroll
        for (int u = 0; u < 8; ++u) d[u] = __bfloat162float(z8[u]) > 0.0f ? gg[u] : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) dZt[(c0 + u) * kLd64 + r] = __float2bfloat16_rn(d[u]);
    }
    if (threadIdx.x < kTM) {
      const int i = base + threadIdx.x;
      float f[kF];
      if (i < in.n) features(in, i, f);
      else
        for (int k = 0; k < kF; ++k) f[k] = 0.0f;
      for (int k = 0; k < kF; ++k) Ft[k * kLd64 + threadIdx.x] = __float2bfloat16_rn(f[k]);
    }
    __syncthreads();
    warp_gemm<kTM, 2, kLd64, kLd64>(dZt + w * 16 * kLd64, Ft, acc);
    if (threadIdx.x < kW)
      for (int r = 0; r < kTM; ++r) db += __bfloat162float(dZt[threadIdx.x * kLd64 + r]);
  }
  float* out = part + (int64_t)blockIdx.x * kPartStride;
#pragma unroll
  for (int nt = 0; nt < 2; ++nt)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int o = w * 16 + g + 8 * h, c = nt * 8 + t * 2;
      out[o * kF + c] = acc[nt][2 * h];
      out[o * kF + c + 1] = acc[nt][2 * h + 1];
    }
  if (threadIdx.x < kW) out[kW * kF + threadIdx.x] = db;
}

// grad[k] = sum over blocks b (ascending) of part[b * stride + k]
__global__ void k_gnn_reduce(const float* __restrict__ part, int nblk, int stride, int count, float* __restrict__ out) {
  note_launch();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * stride + k];
    out[k] = (float)s;
  }
}

// Adam on the FP32 master weights, then the BF16 copies.
__global__ void k_gnn_adam(int count, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, bf16* __restrict__ wb, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
  note_launch();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.0f - b1) * gk;
    const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    const float wk = w[k] - lr * (mk / c1) / (sqrtf(vk / c2) + eps);
    w[k] = wk;
    wb[k] = __float2bfloat16_rn(wk);
  }
}

__global__ void k_gnn_cast(int count, const float* __restrict__ w, bf16* __restrict__ wb) {
  note_launch();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x)
    wb[k] = __float2bfloat16_rn(w[k]);
}

}  // namespace
}  // namespace fl

using namespace fl;

struct fl_gnn_t {
  fl_mesh_t* m = nullptr;
  int n = 0;
  DevBuf<float> w, g, am, av, inv_deg, dH, dH2, dA, part, scal;
  DevBuf<bf16> wb, H, Z, A;  // H, Z: 4 x n x 64; A: 3 x n x 64
  int steps = 0;
  float nact_inv = 0.0f;
  const double* kval = nullptr;  // matrix of the energy-norm loss (null: squared error)
  DevBuf<double> e, Ke;
};

namespace {

bf16* Hbuf(fl_gnn_t* G, int l) { return G->H.p + (size_t)l * G->n * kW; }
bf16* Zbuf(fl_gnn_t* G, int l) { return G->Z.p + (size_t)l * G->n * kW; }
bf16* Abuf(fl_gnn_t* G, int l) { return G->A.p + (size_t)l * G->n * kW; }

unsigned tile_grid(int n) {
  const int ntiles = (n + kTM - 1) / kTM;
  return (unsigned)std::max(1, std::min(ntiles, num_sms() * 8));
}
unsigned persist_grid(int n) {
  const int ntiles = (n + kTM - 1) / kTM;
  return (unsigned)std::max(1, std::min(ntiles, kPersist));
}
unsigned warp_grid(int n) { return grid_for((int64_t)n * 32, 256, 8); }

int forward(fl_gnn_t* G, const double* p1, const double* p2, const double* b, double* pred, const double* target,
            const uint8_t* mask, cudaStream_t s) {
  const int n = G->n;
  fl_mesh_t* m = G->m;
  FL_TRY_CUDA(cudaMemsetAsync(G->scal.p, 0, sizeof(float) * 4, s));
  k_gnn_scales<<<grid_for(n, 256, 4), 256, 0, s>>>(n, p1, b, G->scal.p);
  Inputs in{n, p1, p2, b, m->coords.p, G->scal.p};
  const bool train = target != nullptr;
  k_gnn_encode<<<tile_grid(n), kTh, 0, s>>>(in, G->wb.p + kOffWe, G->w.p + kOffBe, train ? Zbuf(G, 0) : nullptr,
                                            Hbuf(G, 0));
  for (int l = 1; l <= kLayers; ++l) {
    const int off = kOffL + (l - 1) * kLayerSize;
    k_gnn_layer_fwd<<<tile_grid(n), kTh, 0, s>>>(n, m->findrm.p, m->colm.p, G->inv_deg.p, Hbuf(G, l - 1),
                                                  G->wb.p + off, G->w.p + off + 2 * kW * kW,
                                                  train ? Abuf(G, l - 1) : nullptr, train ? Zbuf(G, l) : nullptr,
                                                  Hbuf(G, l));
  }
  const bool energy = train && G->kval;
  DecodeArgs D{in, Hbuf(G, kLayers), G->wb.p + kOffWd, G->w.p + kOffBd, pred, target, mask, G->nact_inv,
               G->dH.p, G->part.p, energy ? 1 : 0, G->e.p, nullptr};
  k_gnn_decode<<<persist_grid(n), kTh, 0, s>>>(D);
  if (energy) {
    FL_TRY(csr_mult(m, G->kval, G->e.p, G->Ke.p, s));
    D.pred = nullptr;
    D.Ke = G->Ke.p;
    k_gnn_decode<<<persist_grid(n), kTh, 0, s>>>(D);
  }
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

// Gradients of the loss into G->g (forward with target first).
int backward(fl_gnn_t* G, const double* p1, const double* p2, const double* b, cudaStream_t s) {
  const int n = G->n;
  fl_mesh_t* m = G->m;
  const unsigned pg = persist_grid(n);
  // decoder partials -> grad[wd], grad[bd], loss (scal[2])
  k_gnn_reduce<<<1, 128, 0, s>>>(G->part.p, (int)persist_grid(n), kW + 2, kW + 1, G->g.p + kOffWd);
  k_gnn_reduce<<<1, 32, 0, s>>>(G->part.p + kW + 1, (int)persist_grid(n), kW + 2, 1, G->scal.p + 2);
  float* cur = G->dH.p;
  float* nxt = G->dH2.p;
  for (int l = kLayers; l >= 1; --l) {
    const int off = kOffL + (l - 1) * kLayerSize;
    k_gnn_bwd_dx<<<tile_grid(n), kTh, 0, s>>>(n, cur, Zbuf(G, l), G->wb.p + off, nxt, G->dA.p);
    k_gnn_bwd_dw<<<pg, kThW, 0, s>>>(n, cur, Zbuf(G, l), Hbuf(G, l - 1), Abuf(G, l - 1), G->part.p);
    k_gnn_reduce<<<grid_for(kLayerSize, 256, 4), 256, 0, s>>>(G->part.p, (int)pg, kPartStride, kLayerSize,
                                                               G->g.p + off);
    k_gnn_agg_bwd<<<warp_grid(n), 256, 0, s>>>(n, m->findrm.p, m->colm.p, G->inv_deg.p, G->dA.p, nxt);
    std::swap(cur, nxt);
  }
  Inputs in{n, p1, p2, b, m->coords.p, G->scal.p};
  k_gnn_bwd_enc<<<pg, kTh, 0, s>>>(in, cur, Zbuf(G, 0), G->part.p);
  k_gnn_reduce<<<grid_for(kW * kF + kW, 256, 4), 256, 0, s>>>(G->part.p, (int)pg, kPartStride, kW * kF + kW,
                                                               G->g.p + kOffWe);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

int set_mask(fl_gnn_t* G, const uint8_t* mask, int32_t nact) {
  FL_CHECK_ARG(nact > 0 || !mask, "active node count");
  G->nact_inv = 1.0f / (float)(mask ? nact : G->n);
  return FL_OK;
}

}  // namespace

extern "C" int fl_gnn_num_params(void) { return kParams; }

extern "C" int fl_gnn_create(fl_mesh mesh, fl_gnn* out) {
  FL_CHECK_ARG(mesh && out, "null argument");
  FL_CHECK_ARG(mesh->loc == 4, "the network runs on P1 meshes (nodes are the coordinate vertices)");
  FL_CHECK_ARG(mesh->N == mesh->Nx, "P1 field mesh and coordinates must share nodes");
  fl_gnn_t* G = new fl_gnn_t();
  G->m = mesh;
  G->n = mesh->N;
  const size_t nw = (size_t)G->n * kW;
  int st = FL_OK;
  do {
    if ((st = G->w.reserve(kParams)) || (st = G->g.reserve(kParams)) || (st = G->am.reserve(kParams)) ||
        (st = G->av.reserve(kParams)) || (st = G->wb.reserve(kParams)) || (st = G->inv_deg.reserve(G->n)) ||
        (st = G->dH.reserve(nw)) || (st = G->dH2.reserve(nw)) || (st = G->dA.reserve(nw)) ||
        (st = G->part.reserve((size_t)kPersist * kPartStride)) || (st = G->scal.reserve(4)) ||
        (st = G->H.reserve(nw * (kLayers + 1))) || (st = G->Z.reserve(nw * (kLayers + 1))) ||
        (st = G->A.reserve(nw * kLayers)))
      break;
    cudaStream_t s = mesh->stream;
    if (cudaMemsetAsync(G->w.p, 0, sizeof(float) * kParams, s) != cudaSuccess ||
        cudaMemsetAsync(G->am.p, 0, sizeof(float) * kParams, s) != cudaSuccess ||
        cudaMemsetAsync(G->av.p, 0, sizeof(float) * kParams, s) != cudaSuccess) {
      st = FL_ERR_CUDA;
      break;
    }
    k_gnn_cast<<<grid_for(kParams, 256, 4), 256, 0, s>>>(kParams, G->w.p, G->wb.p);
    k_gnn_inv_deg<<<grid_for(G->n, 256, 4), 256, 0, s>>>(G->n, mesh->findrm.p, G->inv_deg.p);
    if (cudaStreamSynchronize(s) != cudaSuccess) st = FL_ERR_CUDA;
  } while (0);
  if (st != FL_OK) {
    delete G;
    if (st == FL_ERR_CUDA) set_error("network allocation: %s", cudaGetErrorString(cudaGetLastError()));
    return st;
  }
  *out = G;
  return FL_OK;
}

extern "C" int fl_gnn_destroy(fl_gnn G) {
  if (G) {
    cudaDeviceSynchronize();
    delete G;
  }
  return FL_OK;
}

extern "C" int fl_gnn_set_loss(fl_gnn G, const double* val) {
  FL_CHECK_ARG(G, "null network");
  if (val) {
    FL_TRY(G->e.reserve(G->n));
    FL_TRY(G->Ke.reserve(G->n));
  }
  G->kval = val;
  return FL_OK;
}

extern "C" int fl_gnn_set_weights(fl_gnn G, const float* w, int32_t count) {
  FL_CHECK_ARG(G && w, "null argument");
  FL_CHECK_ARG(count == kParams, "parameter count");
  cudaStream_t s = G->m->stream;
  FL_TRY_CUDA(cudaMemcpyAsync(G->w.p, w, sizeof(float) * kParams, cudaMemcpyHostToDevice, s));
  FL_TRY_CUDA(cudaMemsetAsync(G->am.p, 0, sizeof(float) * kParams, s));
  FL_TRY_CUDA(cudaMemsetAsync(G->av.p, 0, sizeof(float) * kParams, s));
  k_gnn_cast<<<grid_for(kParams, 256, 4), 256, 0, s>>>(kParams, G->w.p, G->wb.p);
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  G->steps = 0;
  return FL_OK;
}

extern "C" int fl_gnn_get_weights(fl_gnn G, float* w, int32_t count) {
  FL_CHECK_ARG(G && w, "null argument");
  FL_CHECK_ARG(count == kParams, "parameter count");
  FL_TRY_CUDA(cudaMemcpy(w, G->w.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
  return FL_OK;
}

extern "C" int fl_gnn_predict(fl_gnn G, const double* p1, const double* p2, const double* b, double* pred,
                              void* stream) {
  FL_CHECK_ARG(G && p1 && p2 && b && pred, "null argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : G->m->stream;
  return forward(G, p1, p2, b, pred, nullptr, nullptr, s);
}

extern "C" int fl_gnn_gradients(fl_gnn G, const double* p1, const double* p2, const double* b,
                                const double* target, const uint8_t* mask, int32_t nact, float* grad,
                                float* loss, void* stream) {
  FL_CHECK_ARG(G && p1 && p2 && b && target && grad, "null argument");
  FL_TRY(set_mask(G, mask, nact));
  cudaStream_t s = stream ? (cudaStream_t)stream : G->m->stream;
  FL_TRY(forward(G, p1, p2, b, nullptr, target, mask, s));
  FL_TRY(backward(G, p1, p2, b, s));
  FL_TRY_CUDA(cudaMemcpyAsync(grad, G->g.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost, s));
  float sc[4];
  FL_TRY_CUDA(cudaMemcpyAsync(sc, G->scal.p, sizeof(float) * 4, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  if (loss) *loss = sc[2] * G->nact_inv;
  return FL_OK;
}

extern "C" int fl_gnn_train_step(fl_gnn G, const double* p1, const double* p2, const double* b,
                                 const double* target, const uint8_t* mask, int32_t nact, float lr,
                                 float* loss_dev, void* stream) {
  FL_CHECK_ARG(G && p1 && p2 && b && target, "null argument");
  FL_CHECK_ARG(lr >= 0.0f, "learning rate");
  FL_TRY(set_mask(G, mask, nact));
  cudaStream_t s = stream ? (cudaStream_t)stream : G->m->stream;
  FL_TRY(forward(G, p1, p2, b, nullptr, target, mask, s));
  FL_TRY(backward(G, p1, p2, b, s));
  G->steps += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f - powf(b1, (float)G->steps), c2 = 1.0f - powf(b2, (float)G->steps);
  k_gnn_adam<<<grid_for(kParams, 256, 4), 256, 0, s>>>(kParams, G->w.p, G->g.p, G->am.p, G->av.p, G->wb.p, lr,
                                                        b1, b2, 1e-8f, c1, c2);
  // loss_dev (device, optional): sum of squared normalised errors of this step
  if (loss_dev) FL_TRY_CUDA(cudaMemcpyAsync(loss_dev, G->scal.p + 2, sizeof(float), cudaMemcpyDeviceToDevice, s));
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}
