// Learned continuation predictor: an edge message-passing network that reads
// the newest converged states and the mesh geometry and predicts how to
// extrapolate to the next parameter value; trained online on the states the
// continuation itself converges to.
//
// Network (hidden width 64, 3 message-passing layers):
//   x_i   = [Re/Im psi_k, Re/Im s~, Re/Im q~, Re/Im c~, mu_new, 1]     (10)
//           s = psi_k - psi_{k-1}, q = quadratic - secant extrapolation,
//           c = cubic - quadratic extrapolation (phase aligned), ~ = / rms
//   e_ij  = [alpha_e / mean|alpha|, +-p_e / rms p, |e| / mean|e|, 1]  (4)
//   h0    = relu(x W_enc + b_enc)
//   layer: A = h W_a, B = h W_b,
//          M_i = sum_j relu(A_i + B_j + e_ij W_c + b_m),
//          h  <- h + relu([h, M] W_u + b_u)
//   z     = mean_i h_i; w = relu(z W_r1 + b_r1) W_r2 + b_r2   (a scalar)
//   prediction = quadratic + w c  (w = 0: quadratic, w = 1: cubic
//   extrapolation; the readout starts near the cubic)
// The readout is global: the correction is a multiple of a smooth
// history-difference field, so node-level rounding noise (which the KEO
// amplifies) never enters the predicted state, and an error in w is scaled
// by |c|, the difference of two extrapolants.  The loss is the linearised
// residual of the prediction relative to the quadratic's: with d = target -
// quadratic and J the Jacobian at the phase-aligned target,
// F(quadratic + w c) ~ J (w c - d), and the loss ||J(w c - d)||^2 / ||J d||^2
// is exact from the three Gram scalars of (J c, J d).
// Node GEMMs run on the tensor cores with BF16 operands and FP32
// accumulation (mma.sync m16n8k16); the message operands A, B are stored in
// FP16 and the forward messages are formed and summed in packed FP16
// arithmetic (two channels per instruction); the backward pass, weight
// gradients (tensor cores, FP32 accumulation) and the optimiser are FP32.
// Every reduction is deterministic (block partials summed in a fixed order).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <vector>

#include "mpnn.cuh"
#include "spmv.cuh"

namespace nosh {

using namespace dev;

namespace {

constexpr int H = 64;      // hidden width
constexpr int FX = 10;     // node input features
constexpr int RH = 32;     // readout hidden width
constexpr int FE = 4;      // edge features
constexpr int LAYERS = 3;

// flat parameter layout (FP32 master copy)
struct Layout {
  int64_t enc_w, enc_b, r1_w, r1_b, r2_w, r2_b, total;
  int64_t wa[LAYERS], wb[LAYERS], wc[LAYERS], bm[LAYERS], wu[LAYERS], bu[LAYERS];
  Layout() {
    int64_t o = 0;
    enc_w = o; o += FX * H;
    enc_b = o; o += H;
    for (int l = 0; l < LAYERS; l++) {
      wa[l] = o; o += H * H;
      wb[l] = o; o += H * H;
      wc[l] = o; o += FE * H;
      bm[l] = o; o += H;
      wu[l] = o; o += 2 * H * H;
      bu[l] = o; o += H;
    }
    r1_w = o; o += H * RH;
    r1_b = o; o += RH;
    r2_w = o; o += RH;
    r2_b = o; o += 1;
    total = o;
  }
};

// ------------------------------------------------ tensor-core node GEMM
// out[r, 0:64] (=, +=) [in0[r, 0:K0], in1[r, 0:K1]] @ W, W stored as
// Wt[64][K] BF16 (transposed, K = K0 + K1 <= 128, K0, K1 multiples of 16
// or K1 = 0).  One warp per 16 rows, 4 warps per CTA.  Used by the backward
// pass (the forward runs in the fused layer kernels below).
enum Epi { EPI_LINEAR = 0, EPI_ACCUM = 1 };

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <int EPI>
__global__ void __launch_bounds__(128) gemm64_kernel(int64_t n, const float *__restrict__ in0, int K0,
                                                     const float *__restrict__ in1, int K1,
                                                     const __nv_bfloat16 *__restrict__ Wt,
                                                     float *__restrict__ out) {
  constexpr int KMAX = 128, LD = KMAX + 8;  // padded rows: conflict-free
  __shared__ __align__(16) __nv_bfloat16 sW[H * LD];
  const int K = K0 + K1;
  for (int q = threadIdx.x; q < H * K; q += blockDim.x) sW[(q / K) * LD + (q % K)] = Wt[q];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int64_t r0 = (blockIdx.x * 4 + warp) * 16;
  if (r0 >= n) return;
  const int64_t ra = r0 + g, rb = r0 + g + 8;
  float acc[8][4];
#pragma unroll
  for (int t = 0; t < 8; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
  for (int kk = 0; kk < K; kk += 16) {
    const float *src = kk < K0 ? in0 : in1;
    const int ld = kk < K0 ? K0 : K1, kc = kk < K0 ? kk : kk - K0;
    float2 a[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    if (ra < n) {
      a[0] = *reinterpret_cast<const float2 *>(src + ra * ld + kc + tig * 2);
      a[2] = *reinterpret_cast<const float2 *>(src + ra * ld + kc + tig * 2 + 8);
    }
    if (rb < n) {
      a[1] = *reinterpret_cast<const float2 *>(src + rb * ld + kc + tig * 2);
      a[3] = *reinterpret_cast<const float2 *>(src + rb * ld + kc + tig * 2 + 8);
    }
    const uint32_t a0 = pack_bf16(a[0].x, a[0].y), a1 = pack_bf16(a[1].x, a[1].y);
    const uint32_t a2 = pack_bf16(a[2].x, a[2].y), a3 = pack_bf16(a[3].x, a[3].y);
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const __nv_bfloat16 *w = sW + (t * 8 + g) * LD + kk + tig * 2;
      const uint32_t b0 = *reinterpret_cast<const uint32_t *>(w);
      const uint32_t b1 = *reinterpret_cast<const uint32_t *>(w + 8);
      mma_bf16(acc[t], a0, a1, a2, a3, b0, b1);
    }
  }
#pragma unroll
  for (int t = 0; t < 8; t++) {
    const int c = t * 8 + tig * 2;
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int64_t r = half ? rb : ra;
      if (r >= n) continue;
      const float v0 = acc[t][2 * half], v1 = acc[t][2 * half + 1];
      float2 *o = reinterpret_cast<float2 *>(out + r * H + c);
      if (EPI == EPI_LINEAR) {
        *o = make_float2(v0, v1);
      } else {
        const float2 p = *o;
        *o = make_float2(p.x + v0, p.y + v1);
      }
    }
  }
}

// forward operand: W (K x ncols, row-major FP32 inside the parameter
// vector) -> Wt[64][K] BF16 with Wt[n][k] = W[k][col0 + n]
__global__ void to_bf16_t(const float *__restrict__ W, int K, int ncols, int col0, __nv_bfloat16 *__restrict__ Wt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= H * K) return;
  const int n = q / K, k = q % K;
  Wt[q] = __float2bfloat16(W[(int64_t)k * ncols + col0 + n]);
}

// encoder operand: Wt[n][k] = W[k][n] for k < 8, zero for the padding k < 16
__global__ void enc_to_bf16(const float *__restrict__ W, __nv_bfloat16 *__restrict__ Wt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= H * 16) return;
  const int n = q / 16, k = q % 16;
  Wt[q] = __float2bfloat16(k < FX ? W[k * H + n] : 0.f);
}

__global__ void to_bf16_rows(const float *__restrict__ W, int rows, int row0, __nv_bfloat16 *__restrict__ Wt) {
  // Wt[n][k] = W[row0 + n][k] for a row-major [* x 64] W: the operand of
  // dIn[:, row0:row0+64] = dOut @ W[row0:row0+64, :]^T
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= H * H) return;
  const int n = q / H, k = q % H;
  Wt[q] = __float2bfloat16(W[(int64_t)(row0 + n) * H + k]);
  (void)rows;
}

// ------------------------------------------------- fused forward layers
// A CTA of 4 warps owns tiles of 64 consecutive rows (16 per warp); each CTA
// walks a contiguous range of tiles, so the neighbour rows a tile gathers
// (mesh-ordered graphs: bands at fixed index offsets) are largely the rows
// its previous tiles gathered.  Per tile and warp, the FP32 16 x 64 state
// lives in registers in the mma accumulator layout: v[t][0..1] = row g,
// columns 8t + 2q, 8t + 2q + 1; v[t][2..3] = the same columns of row g + 8
// (g = lane / 4, q = lane % 4), which is also the A-operand layout of the
// next m16n8k16 (k-step kk takes column tiles 2kk and 2kk + 1).
constexpr int TILE = 64;
constexpr int LDU = 2 * H + 8;  // smem row strides (BF16), padded: conflict-free fragment loads
constexpr int LDAB = H + 8;
constexpr int LDM = H + 8;
constexpr int LDE = 16 + 8;
constexpr size_t kLayerSmem = (size_t)(H * LDU + 2 * H * LDAB + 4 * 16 * LDM) * sizeof(__nv_bfloat16) +
                              4 * H * sizeof(float);
constexpr size_t kEncSmem = (size_t)(H * LDE + 2 * H * LDAB) * sizeof(__nv_bfloat16);
// the update-only layer (M from global memory): no M staging
constexpr size_t kUpdateSmem = (size_t)(H * LDU + 2 * H * LDAB) * sizeof(__nv_bfloat16) + 4 * H * sizeof(float);

__device__ __forceinline__ void frag_from_c(const float (&v)[8][4], int kk, uint32_t &a0, uint32_t &a1,
                                            uint32_t &a2, uint32_t &a3) {
  a0 = pack_bf16(v[2 * kk][0], v[2 * kk][1]);
  a1 = pack_bf16(v[2 * kk][2], v[2 * kk][3]);
  a2 = pack_bf16(v[2 * kk + 1][0], v[2 * kk + 1][1]);
  a3 = pack_bf16(v[2 * kk + 1][2], v[2 * kk + 1][3]);
}

// BF16 [rows][K] (global, K a multiple of 8) -> smem rows of stride ld
__device__ __forceinline__ void stage_w(__nv_bfloat16 *dst, const __nv_bfloat16 *__restrict__ src, int rows, int K,
                                        int ld) {
  const int per_row = K / 8;
  for (int q = threadIdx.x; q < rows * per_row; q += blockDim.x) {
    const int r = q / per_row, k = (q % per_row) * 8;
    *reinterpret_cast<uint4 *>(dst + r * ld + k) = *reinterpret_cast<const uint4 *>(src + r * K + k);
  }
}

// [A | B] = bf16(v) @ [W_a | W_b] for the warp's 16 rows; FP16 stores (the
// message operands, added in packed FP16 arithmetic by the aggregation)
__device__ __forceinline__ void emit_ab(const float (&v)[8][4], const __nv_bfloat16 *sW, int64_t ra, int64_t rb,
                                        int64_t n, __half *__restrict__ A, __half *__restrict__ B, int g, int q) {
#pragma unroll
  for (int part = 0; part < 2; part++) {
    float acc[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      uint32_t a0, a1, a2, a3;
      frag_from_c(v, kk, a0, a1, a2, a3);
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const __nv_bfloat16 *w = sW + (part * H + t * 8 + g) * LDAB + kk * 16 + q * 2;
        mma_bf16(acc[t], a0, a1, a2, a3, *reinterpret_cast<const uint32_t *>(w),
                 *reinterpret_cast<const uint32_t *>(w + 8));
      }
    }
    __half *dst = part ? B : A;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int c = t * 8 + q * 2;
      if (ra < n) *reinterpret_cast<__half2 *>(dst + ra * H + c) = __floats2half2_rn(acc[t][0], acc[t][1]);
      if (rb < n) *reinterpret_cast<__half2 *>(dst + rb * H + c) = __floats2half2_rn(acc[t][2], acc[t][3]);
    }
  }
}

__device__ __forceinline__ void tile_range(int64_t tiles, int64_t &t0, int64_t &t1) {
  t0 = tiles * blockIdx.x / gridDim.x;
  t1 = tiles * (blockIdx.x + 1) / gridDim.x;
}

// h0 = relu(X W_enc + b_enc) (X: n x 10, K padded to 16 with zeros), then
// layer 0's A, B
__global__ void __launch_bounds__(128) encode_kernel(int64_t n, const float *__restrict__ X,
                                                     const __nv_bfloat16 *__restrict__ We,
                                                     const float *__restrict__ be,
                                                     const __nv_bfloat16 *__restrict__ Wab, float *__restrict__ h,
                                                     __half *__restrict__ A, __half *__restrict__ B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *sWe = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
  __nv_bfloat16 *sWab = sWe + H * LDE;
  stage_w(sWe, We, H, 16, LDE);
  stage_w(sWab, Wab, 2 * H, H, LDAB);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  int64_t t0, t1;
  tile_range((n + TILE - 1) / TILE, t0, t1);
  for (int64_t tile = t0; tile < t1; tile++) {
    const int64_t r0 = tile * TILE + warp * 16;
    if (r0 >= n) continue;
    const int64_t ra = r0 + g, rb = r0 + g + 8;
    float2 x[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    // columns 2q, 2q + 1 (< 8) and 8 + 2q, 9 + 2q (only q = 0 is < FX = 10)
    if (ra < n) {
      x[0] = *reinterpret_cast<const float2 *>(X + ra * FX + 2 * q);
      if (q == 0) x[2] = *reinterpret_cast<const float2 *>(X + ra * FX + 8);
    }
    if (rb < n) {
      x[1] = *reinterpret_cast<const float2 *>(X + rb * FX + 2 * q);
      if (q == 0) x[3] = *reinterpret_cast<const float2 *>(X + rb * FX + 8);
    }
    const uint32_t a0 = pack_bf16(x[0].x, x[0].y), a1 = pack_bf16(x[1].x, x[1].y);
    const uint32_t a2 = pack_bf16(x[2].x, x[2].y), a3 = pack_bf16(x[3].x, x[3].y);
    float v[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
      v[t][0] = v[t][1] = v[t][2] = v[t][3] = 0.f;
      const __nv_bfloat16 *w = sWe + (t * 8 + g) * LDE + q * 2;
      mma_bf16(v[t], a0, a1, a2, a3, *reinterpret_cast<const uint32_t *>(w),
               *reinterpret_cast<const uint32_t *>(w + 8));
    }
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int c = t * 8 + q * 2;
      const float b0 = be[c], b1 = be[c + 1];
      v[t][0] = ra < n ? fmaxf(v[t][0] + b0, 0.f) : 0.f;
      v[t][1] = ra < n ? fmaxf(v[t][1] + b1, 0.f) : 0.f;
      v[t][2] = rb < n ? fmaxf(v[t][2] + b0, 0.f) : 0.f;
      v[t][3] = rb < n ? fmaxf(v[t][3] + b1, 0.f) : 0.f;
      if (ra < n) *reinterpret_cast<float2 *>(h + ra * H + c) = make_float2(v[t][0], v[t][1]);
      if (rb < n) *reinterpret_cast<float2 *>(h + rb * H + c) = make_float2(v[t][2], v[t][3]);
    }
    emit_ab(v, sWab, ra, rb, n, A, B, g, q);
  }
}

// Per-lane message constants: W_c rows 0..2 for the lane's 4 channels
// (packed FP16) and b_m + W_c[3] (the constant edge feature folded in).
struct MsgConst {
  __half2 w2[3][2];
  float abias[4];
};

__device__ __forceinline__ void msg_const(const float *__restrict__ Wc, const float *__restrict__ bm, int c4,
                                          MsgConst &k) {
#pragma unroll
  for (int f = 0; f < 3; f++) {
    const float4 w = *reinterpret_cast<const float4 *>(Wc + f * H + c4);
    k.w2[f][0] = __floats2half2_rn(w.x, w.y);
    k.w2[f][1] = __floats2half2_rn(w.z, w.w);
  }
  const float4 b = *reinterpret_cast<const float4 *>(bm + c4);
  const float4 w3 = *reinterpret_cast<const float4 *>(Wc + 3 * H + c4);
  k.abias[0] = b.x + w3.x;
  k.abias[1] = b.y + w3.y;
  k.abias[2] = b.z + w3.z;
  k.abias[3] = b.w + w3.w;
}

// M_r for the lane's 4 channels (c4 = 4 (lane % 16)); a half-warp per row,
// both halves of the warp call together (the neighbour shuffles span the
// warp); rows r >= n give zeros.  Packed FP16 message arithmetic: a = A_r +
// b_m + W_c[3], two channels per instruction; the 16 neighbour gathers of a
// batch are unconditional (row 0 stands in for missing neighbours, masked
// out of the sum) so all are in flight at once.
__device__ __forceinline__ void aggregate_row(int64_t r, int64_t n, const int32_t *__restrict__ rp,
                                              const int32_t *__restrict__ ci, const float4 *__restrict__ ef,
                                              const __half *__restrict__ A, const __half *__restrict__ B,
                                              const MsgConst &k, int hl, int half, int c4, float (&m)[4]) {
  const __half2 zero2 = __float2half2_rn(0.f);
  int32_t beg = 0, deg = 0;
  __half2 a2[2] = {zero2, zero2}, m2[2] = {zero2, zero2};
  if (r < n) {
    beg = rp[r];
    deg = rp[r + 1] - beg;
    const uint2 av = *reinterpret_cast<const uint2 *>(A + r * H + c4);
    const float2 a01 = __half22float2(*reinterpret_cast<const __half2 *>(&av.x));
    const float2 a23 = __half22float2(*reinterpret_cast<const __half2 *>(&av.y));
    a2[0] = __floats2half2_rn(a01.x + k.abias[0], a01.y + k.abias[1]);
    a2[1] = __floats2half2_rn(a23.x + k.abias[2], a23.y + k.abias[3]);
  }
  const int maxdeg = max(deg, __shfl_xor_sync(0xffffffffu, deg, 16));
  for (int k0 = 0; k0 < maxdeg; k0 += 16) {
    // each lane fetches one neighbour index and its edge features
    const bool ok = k0 + hl < deg;
    const int32_t jl = ok ? ci[beg + k0 + hl] : 0;
    const float4 el = ok ? ef[beg + k0 + hl] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int cnt = deg - k0;  // this half's remaining neighbours (may be <= 0)
    uint2 bv[16];
#pragma unroll
    for (int u = 0; u < 16; u++) {
      const int32_t j = __shfl_sync(0xffffffffu, jl, (half << 4) + u);
      bv[u] = *reinterpret_cast<const uint2 *>(B + (int64_t)j * H + c4);
    }
#pragma unroll
    for (int u = 0; u < 16; u++) {
      const int src = (half << 4) + u;
      const __half2 ex = __float2half2_rn(__shfl_sync(0xffffffffu, el.x, src));
      const __half2 ey = __float2half2_rn(__shfl_sync(0xffffffffu, el.y, src));
      const __half2 ez = __float2half2_rn(__shfl_sync(0xffffffffu, el.z, src));
      const __half2 *bb = reinterpret_cast<const __half2 *>(&bv[u]);
      const bool live = u < cnt;
#pragma unroll
      for (int cc = 0; cc < 2; cc++) {
        __half2 pv = __hadd2(a2[cc], bb[cc]);
        pv = __hfma2(ex, k.w2[0][cc], pv);
        pv = __hfma2(ey, k.w2[1][cc], pv);
        pv = __hfma2(ez, k.w2[2][cc], pv);
        if (live) m2[cc] = __hadd2(m2[cc], __hmax2(pv, zero2));
      }
    }
  }
  const float2 m01 = __half22float2(m2[0]), m23 = __half22float2(m2[1]);
  m[0] = m01.x;
  m[1] = m01.y;
  m[2] = m23.x;
  m[3] = m23.y;
}

// Inference split of a layer: the aggregation alone, at high occupancy (the
// fused layer holds 12 warps per SM and waits on the gathers), writing M in
// BF16 (the update GEMM's operand, rounded as the fused layer rounds it).
__global__ void __launch_bounds__(256, 4) mp_aggregate_kernel(int64_t n, const int32_t *__restrict__ rp,
                                                           const int32_t *__restrict__ ci,
                                                           const float4 *__restrict__ ef,
                                                           const __half *__restrict__ A,
                                                           const __half *__restrict__ B,
                                                           const float *__restrict__ Wc,
                                                           const float *__restrict__ bm,
                                                           __nv_bfloat16 *__restrict__ Mb) {
  const int lane = threadIdx.x & 31, hl = lane & 15, half = lane >> 4, c4 = hl * 4;
  MsgConst k;
  msg_const(Wc, bm, c4, k);
  // each CTA walks one contiguous range of rows, 16 at a time (a half-warp
  // per row): the neighbours of nearby rows (mesh-ordered graphs: bands at
  // fixed index offsets) are then largely in this SM's L1
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5;
  const int64_t per = ((n + gridDim.x - 1) / gridDim.x + 1) & ~(int64_t)1;
  const int64_t beg = blockIdx.x * per, end = beg + per < n ? beg + per : n;
  // warp-uniform loop over row pairs
  for (int64_t r0 = beg + 2 * w; r0 < end; r0 += 2 * wpc) {
    const int64_t r = r0 + half;
    float m[4];
    aggregate_row(r, end, rp, ci, ef, A, B, k, hl, half, c4, m);
    if (r < end) {
      uint2 mv;
      *reinterpret_cast<__nv_bfloat162 *>(&mv.x) = __floats2bfloat162_rn(m[0], m[1]);
      *reinterpret_cast<__nv_bfloat162 *>(&mv.y) = __floats2bfloat162_rn(m[2], m[3]);
      *reinterpret_cast<uint2 *>(Mb + r * H + c4) = mv;
    }
  }
}

// One message-passing layer:
//   M_i = sum_j relu(A_i + B_j + e_ij W_c + b_m)          (FP32 sums)
//   R   = relu(bf16([h, M]) @ bf16(W_u) + b_u),  h' = h + R
// then, for all but the last layer, the next layer's A, B from h'; the last
// layer writes per-CTA column sums of h' (the mean-pool partials) instead of
// h'.  TRAIN also stores M and R (FP32) for the backward pass.  PRE_M (the
// inference split): M comes from mp_aggregate_kernel in BF16 (Mb) and the
// kernel is the update GEMM alone.
template <bool TRAIN, bool LAST, bool PRE_M>
__global__ void __launch_bounds__(128, 3) mp_layer_kernel(
    int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci, const float4 *__restrict__ ef,
    const float *__restrict__ h, const __half *__restrict__ A, const __half *__restrict__ B,
    const float *__restrict__ Wc, const float *__restrict__ bm, const __nv_bfloat16 *__restrict__ Wu,
    const float *__restrict__ bu, const __nv_bfloat16 *__restrict__ Wab, float *__restrict__ h_out,
    __half *__restrict__ A_out, __half *__restrict__ B_out, float *__restrict__ M_out,
    float *__restrict__ R_out, float *__restrict__ pool, const __nv_bfloat16 *__restrict__ Mb) {
  static_assert(!(TRAIN && PRE_M), "training runs the fused layer");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *sWu = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
  __nv_bfloat16 *sWab = sWu + H * LDU;
  __nv_bfloat16 *sM = sWab + 2 * H * LDAB;
  float *sPool = reinterpret_cast<float *>(PRE_M ? sM : sM + 4 * 16 * LDM);
  stage_w(sWu, Wu, H, 2 * H, LDU);
  if (!LAST) stage_w(sWab, Wab, 2 * H, H, LDAB);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  __nv_bfloat16 *sMw = sM + warp * 16 * LDM;
  // aggregation: a half-warp per row, 4 channels per lane
  const int hl = lane & 15, half = lane >> 4, c4 = hl * 4;
  MsgConst mk;
  if (!PRE_M) msg_const(Wc, bm, c4, mk);
  float psum[8][2];
#pragma unroll
  for (int t = 0; t < 8; t++) psum[t][0] = psum[t][1] = 0.f;
  int64_t t0, t1;
  tile_range((n + TILE - 1) / TILE, t0, t1);
  for (int64_t tile = t0; tile < t1; tile++) {
    const int64_t r0 = tile * TILE + warp * 16;
    if (r0 >= n) continue;
    if (!PRE_M) {
      for (int p = 0; p < 8; p++) {
        const int rr = 2 * p + half;
        const int64_t r = r0 + rr;
        float m[4];
        aggregate_row(r, n, rp, ci, ef, A, B, mk, hl, half, c4, m);
        uint2 mv;
        *reinterpret_cast<__nv_bfloat162 *>(&mv.x) = __floats2bfloat162_rn(m[0], m[1]);
        *reinterpret_cast<__nv_bfloat162 *>(&mv.y) = __floats2bfloat162_rn(m[2], m[3]);
        *reinterpret_cast<uint2 *>(sMw + rr * LDM + c4) = mv;
        if (TRAIN && r < n) *reinterpret_cast<float4 *>(M_out + r * H + c4) = make_float4(m[0], m[1], m[2], m[3]);
      }
    }
    __syncwarp();
    // update GEMM: K = 128 = [h (registers) | M (shared memory)]
    const int64_t ra = r0 + g, rb = r0 + g + 8;
    float v[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int c = t * 8 + q * 2;
      const float2 x0 = ra < n ? *reinterpret_cast<const float2 *>(h + ra * H + c) : make_float2(0.f, 0.f);
      const float2 x1 = rb < n ? *reinterpret_cast<const float2 *>(h + rb * H + c) : make_float2(0.f, 0.f);
      v[t][0] = x0.x; v[t][1] = x0.y; v[t][2] = x1.x; v[t][3] = x1.y;
    }
    float acc[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      uint32_t a0, a1, a2, a3;
      frag_from_c(v, kk, a0, a1, a2, a3);
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const __nv_bfloat16 *w = sWu + (t * 8 + g) * LDU + kk * 16 + q * 2;
        mma_bf16(acc[t], a0, a1, a2, a3, *reinterpret_cast<const uint32_t *>(w),
                 *reinterpret_cast<const uint32_t *>(w + 8));
      }
    }
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      uint32_t a0, a1, a2, a3;
      if (PRE_M) {
        // the A-fragment straight from the BF16 rows (zeros past n, as the
        // fused aggregation gives)
        const __nv_bfloat16 *ma = Mb + ra * H + kk * 16 + q * 2, *mb = Mb + rb * H + kk * 16 + q * 2;
        a0 = ra < n ? *reinterpret_cast<const uint32_t *>(ma) : 0u;
        a1 = rb < n ? *reinterpret_cast<const uint32_t *>(mb) : 0u;
        a2 = ra < n ? *reinterpret_cast<const uint32_t *>(ma + 8) : 0u;
        a3 = rb < n ? *reinterpret_cast<const uint32_t *>(mb + 8) : 0u;
      } else {
        const __nv_bfloat16 *mrow = sMw + kk * 16 + q * 2;
        a0 = *reinterpret_cast<const uint32_t *>(mrow + g * LDM);
        a1 = *reinterpret_cast<const uint32_t *>(mrow + (g + 8) * LDM);
        a2 = *reinterpret_cast<const uint32_t *>(mrow + g * LDM + 8);
        a3 = *reinterpret_cast<const uint32_t *>(mrow + (g + 8) * LDM + 8);
      }
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const __nv_bfloat16 *w = sWu + (t * 8 + g) * LDU + H + kk * 16 + q * 2;
        mma_bf16(acc[t], a0, a1, a2, a3, *reinterpret_cast<const uint32_t *>(w),
                 *reinterpret_cast<const uint32_t *>(w + 8));
      }
    }
    __syncwarp();  // sMw is rewritten by the next tile
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int c = t * 8 + q * 2;
      const float b0 = bu[c], b1 = bu[c + 1];
      const float u0 = fmaxf(acc[t][0] + b0, 0.f), u1 = fmaxf(acc[t][1] + b1, 0.f);
      const float u2 = fmaxf(acc[t][2] + b0, 0.f), u3 = fmaxf(acc[t][3] + b1, 0.f);
      v[t][0] = ra < n ? v[t][0] + u0 : 0.f;
      v[t][1] = ra < n ? v[t][1] + u1 : 0.f;
      v[t][2] = rb < n ? v[t][2] + u2 : 0.f;
      v[t][3] = rb < n ? v[t][3] + u3 : 0.f;
      if (TRAIN) {
        if (ra < n) *reinterpret_cast<float2 *>(R_out + ra * H + c) = make_float2(u0, u1);
        if (rb < n) *reinterpret_cast<float2 *>(R_out + rb * H + c) = make_float2(u2, u3);
      }
      if (!LAST) {
        if (ra < n) *reinterpret_cast<float2 *>(h_out + ra * H + c) = make_float2(v[t][0], v[t][1]);
        if (rb < n) *reinterpret_cast<float2 *>(h_out + rb * H + c) = make_float2(v[t][2], v[t][3]);
      }
    }
    if (LAST) {
#pragma unroll
      for (int t = 0; t < 8; t++) {
        psum[t][0] += v[t][0] + v[t][2];
        psum[t][1] += v[t][1] + v[t][3];
      }
    } else {
      emit_ab(v, sWab, ra, rb, n, A_out, B_out, g, q);
    }
  }
  if (LAST) {
    // column sums over the lanes of equal q, then over the 4 warps
#pragma unroll
    for (int t = 0; t < 8; t++)
#pragma unroll
      for (int k = 0; k < 2; k++) {
        float x = psum[t][k];
        x += __shfl_xor_sync(0xffffffffu, x, 4);
        x += __shfl_xor_sync(0xffffffffu, x, 8);
        x += __shfl_xor_sync(0xffffffffu, x, 16);
        psum[t][k] = x;
      }
    if (g == 0)
#pragma unroll
      for (int t = 0; t < 8; t++) {
        sPool[warp * H + t * 8 + q * 2] = psum[t][0];
        sPool[warp * H + t * 8 + q * 2 + 1] = psum[t][1];
      }
    __syncthreads();
    if (threadIdx.x < H)
      pool[(int64_t)blockIdx.x * H + threadIdx.x] =
          (sPool[threadIdx.x] + sPool[H + threadIdx.x]) + (sPool[2 * H + threadIdx.x] + sPool[3 * H + threadIdx.x]);
  }
}

// ------------------------------------------------- edge backward kernels
// Both walk rows with a half-warp per row (4 channels per lane) and gather
// the 16 neighbours of a batch before using any (as the forward layer does).
constexpr int EB_ROWS = 64;  // rows per CTA (16 half-warps x 4)

__device__ __forceinline__ float4 half4_to_float4(uint2 u) {
  const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&u.x));
  const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&u.y));
  return make_float4(a.x, a.y, b.x, b.y);
}

// dA_i = sum_j dM_i [P_ij > 0] (P_ij = A_i + B_j + e_ij W_c + b_m), and the
// CTA's partials of dW_c (4 x 64) and db_m (64): 5 x 64 floats per CTA
__global__ void __launch_bounds__(256) edge_backward_a(int64_t n, const int32_t *__restrict__ rp,
                                                       const int32_t *__restrict__ ci, const float4 *__restrict__ ef,
                                                       const __half *__restrict__ A,
                                                       const __half *__restrict__ B,
                                                       const float *__restrict__ Wc, const float *__restrict__ bm,
                                                       const float *__restrict__ dM, float *__restrict__ dA,
                                                       float *__restrict__ part) {
  __shared__ float red[16][5][H];
  const int lane = threadIdx.x & 31, hw = threadIdx.x >> 4, hl = lane & 15, half = lane >> 4, c4 = hl * 4;
  float wc[FE][4], bmv[4];
#pragma unroll
  for (int f = 0; f < FE; f++) {
    const float4 w = *reinterpret_cast<const float4 *>(Wc + f * H + c4);
    wc[f][0] = w.x; wc[f][1] = w.y; wc[f][2] = w.z; wc[f][3] = w.w;
  }
  {
    const float4 b = *reinterpret_cast<const float4 *>(bm + c4);
    bmv[0] = b.x; bmv[1] = b.y; bmv[2] = b.z; bmv[3] = b.w;
  }
  float gw[5][4];
#pragma unroll
  for (int f = 0; f < 5; f++) gw[f][0] = gw[f][1] = gw[f][2] = gw[f][3] = 0.f;
  for (int rr = 0; rr < EB_ROWS / 16; rr++) {
    const int64_t i = (int64_t)blockIdx.x * EB_ROWS + hw * (EB_ROWS / 16) + rr;
    int32_t beg = 0, deg = 0;
    float a[4] = {0.f, 0.f, 0.f, 0.f}, dm[4] = {0.f, 0.f, 0.f, 0.f};
    if (i < n) {
      beg = rp[i];
      deg = rp[i + 1] - beg;
      const float4 av = half4_to_float4(*reinterpret_cast<const uint2 *>(A + i * H + c4));
      const float4 d = *reinterpret_cast<const float4 *>(dM + i * H + c4);
      a[0] = av.x + bmv[0]; a[1] = av.y + bmv[1]; a[2] = av.z + bmv[2]; a[3] = av.w + bmv[3];
      dm[0] = d.x; dm[1] = d.y; dm[2] = d.z; dm[3] = d.w;
    }
    float sacc[4] = {0.f, 0.f, 0.f, 0.f};
    const int maxdeg = max(deg, __shfl_xor_sync(0xffffffffu, deg, 16));
    for (int k0 = 0; k0 < maxdeg; k0 += 16) {
      const bool ok = k0 + hl < deg;
      const int32_t jl = ok ? ci[beg + k0 + hl] : 0;
      const float4 el = ok ? ef[beg + k0 + hl] : make_float4(0.f, 0.f, 0.f, 0.f);
      const int cnt = deg - k0;
      uint2 bv[16];
#pragma unroll
      for (int u = 0; u < 16; u++) {
        const int32_t j = __shfl_sync(0xffffffffu, jl, (half << 4) + u);
        bv[u] = *reinterpret_cast<const uint2 *>(B + (int64_t)j * H + c4);
      }
#pragma unroll
      for (int u = 0; u < 16; u++) {
        const int src = (half << 4) + u;
        const float e[4] = {__shfl_sync(0xffffffffu, el.x, src), __shfl_sync(0xffffffffu, el.y, src),
                            __shfl_sync(0xffffffffu, el.z, src), __shfl_sync(0xffffffffu, el.w, src)};
        const float4 b = half4_to_float4(bv[u]);
        const float bb[4] = {b.x, b.y, b.z, b.w};
        const bool live = u < cnt;
#pragma unroll
        for (int cc = 0; cc < 4; cc++) {
          const float pv = a[cc] + bb[cc] + e[0] * wc[0][cc] + e[1] * wc[1][cc] + e[2] * wc[2][cc] + e[3] * wc[3][cc];
          const float gg = (live && pv > 0.f) ? dm[cc] : 0.f;
          sacc[cc] += gg;
#pragma unroll
          for (int f = 0; f < FE; f++) gw[f][cc] += e[f] * gg;
          gw[4][cc] += gg;
        }
      }
    }
    if (i < n) *reinterpret_cast<float4 *>(dA + i * H + c4) = make_float4(sacc[0], sacc[1], sacc[2], sacc[3]);
  }
#pragma unroll
  for (int f = 0; f < 5; f++)
#pragma unroll
    for (int cc = 0; cc < 4; cc++) red[hw][f][c4 + cc] = gw[f][cc];
  __syncthreads();
  for (int q = threadIdx.x; q < 5 * H; q += blockDim.x) {
    float t = 0.f;
    for (int w = 0; w < 16; w++) t += red[w][q / H][q % H];
    part[(int64_t)blockIdx.x * 5 * H + q] = t;
  }
}

// dB_j = sum over the rows i that receive from j of dM_i [P_ij > 0]: row j
// of the symmetric graph lists those i; tr[k] is the position of (i, j)
__global__ void __launch_bounds__(256) edge_backward_b(int64_t n, const int32_t *__restrict__ rp,
                                                       const int32_t *__restrict__ ci, const int32_t *__restrict__ tr,
                                                       const float4 *__restrict__ ef,
                                                       const __half *__restrict__ A,
                                                       const __half *__restrict__ B,
                                                       const float *__restrict__ Wc, const float *__restrict__ bm,
                                                       const float *__restrict__ dM, float *__restrict__ dB) {
  const int lane = threadIdx.x & 31, hw = threadIdx.x >> 4, hl = lane & 15, half = lane >> 4, c4 = hl * 4;
  float wc[FE][4], bmv[4];
#pragma unroll
  for (int f = 0; f < FE; f++) {
    const float4 w = *reinterpret_cast<const float4 *>(Wc + f * H + c4);
    wc[f][0] = w.x; wc[f][1] = w.y; wc[f][2] = w.z; wc[f][3] = w.w;
  }
  {
    const float4 b = *reinterpret_cast<const float4 *>(bm + c4);
    bmv[0] = b.x; bmv[1] = b.y; bmv[2] = b.z; bmv[3] = b.w;
  }
  for (int rr = 0; rr < EB_ROWS / 16; rr++) {
    const int64_t j = (int64_t)blockIdx.x * EB_ROWS + hw * (EB_ROWS / 16) + rr;
    int32_t beg = 0, deg = 0;
    float b[4] = {0.f, 0.f, 0.f, 0.f};
    if (j < n) {
      beg = rp[j];
      deg = rp[j + 1] - beg;
      const float4 bv = half4_to_float4(*reinterpret_cast<const uint2 *>(B + j * H + c4));
      b[0] = bv.x + bmv[0]; b[1] = bv.y + bmv[1]; b[2] = bv.z + bmv[2]; b[3] = bv.w + bmv[3];
    }
    float sacc[4] = {0.f, 0.f, 0.f, 0.f};
    const int maxdeg = max(deg, __shfl_xor_sync(0xffffffffu, deg, 16));
    for (int k0 = 0; k0 < maxdeg; k0 += 16) {
      const bool ok = k0 + hl < deg;
      const int32_t il = ok ? ci[beg + k0 + hl] : 0;
      const float4 el = ok ? ef[tr[beg + k0 + hl]] : make_float4(0.f, 0.f, 0.f, 0.f);
      const int cnt = deg - k0;
      uint2 av[16];
      float4 dv[16];
#pragma unroll
      for (int u = 0; u < 16; u++) {
        const int32_t i = __shfl_sync(0xffffffffu, il, (half << 4) + u);
        av[u] = *reinterpret_cast<const uint2 *>(A + (int64_t)i * H + c4);
        dv[u] = *reinterpret_cast<const float4 *>(dM + (int64_t)i * H + c4);
      }
#pragma unroll
      for (int u = 0; u < 16; u++) {
        const int src = (half << 4) + u;
        const float e[4] = {__shfl_sync(0xffffffffu, el.x, src), __shfl_sync(0xffffffffu, el.y, src),
                            __shfl_sync(0xffffffffu, el.z, src), __shfl_sync(0xffffffffu, el.w, src)};
        const float4 ai = half4_to_float4(av[u]);
        const float aa[4] = {ai.x, ai.y, ai.z, ai.w}, dd[4] = {dv[u].x, dv[u].y, dv[u].z, dv[u].w};
        const bool live = u < cnt;
#pragma unroll
        for (int cc = 0; cc < 4; cc++) {
          const float pv = aa[cc] + b[cc] + e[0] * wc[0][cc] + e[1] * wc[1][cc] + e[2] * wc[2][cc] + e[3] * wc[3][cc];
          sacc[cc] += (live && pv > 0.f) ? dd[cc] : 0.f;
        }
      }
    }
    if (j < n) *reinterpret_cast<float4 *>(dB + j * H + c4) = make_float4(sacc[0], sacc[1], sacc[2], sacc[3]);
  }
}

// part[cta][k][c] = sum over the CTA's rows of in[r][k] * dout[r][c] (c <
// 64) and, in row K, sum of dout[r][c] (bias gradient).  in = [in0 | in1].
// part[cta][k][c] = sum over the CTA's rows of in[r][k] * dout[r][c]
// (c < 64) and, in row K, the sum of dout[r][c] (bias gradient);
// in = [in0 | in1], K = K0 + K1 <= 143.  Tensor cores: the reduction over
// rows is the k dimension of m16n8k16 BF16 MMAs (FP32 accumulation), with
// in^T and dout fragments loaded by ldmatrix.trans from row-major tiles of
// 64 rows staged in shared memory; a ones column in the staged input makes
// the bias row.  Each CTA (4 warps) owns a contiguous range of rows and the
// whole (K+1) x 64 output, warps splitting it by 16-feature tiles.
constexpr int WG_TILE = 64;
constexpr int WG_MAXK = 144;
constexpr int WG_LDI = WG_MAXK + 8;  // padded rows: conflict-free ldmatrix
constexpr int WG_LDD = 64 + 8;
constexpr int WG_PARTS = 3 * kNumSMs;

__device__ __forceinline__ void ldsm_x4_trans(uint32_t (&r)[4], const __nv_bfloat16 *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_addr(p)));
}

// rows [r0, r0 + WG_TILE) of an n x width FP32 matrix -> BF16 shared-memory
// columns [col0, col0 + width) (zeros past rend); float4 loads when width is
// a multiple of 4, float2 otherwise (width is even)
__device__ __forceinline__ void stage_rows(__nv_bfloat16 *dst, int ld, int col0, const float *__restrict__ src,
                                           int width, int64_t r0, int64_t rend) {
  if ((width & 3) == 0) {
    const int per = width >> 2;
    for (int q = threadIdx.x; q < WG_TILE * per; q += blockDim.x) {
      const int rr = q / per, c = (q % per) * 4;
      const int64_t r = r0 + rr;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < rend) v = *reinterpret_cast<const float4 *>(src + r * width + c);
      __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(dst + rr * ld + col0 + c);
      o[0] = __floats2bfloat162_rn(v.x, v.y);
      o[1] = __floats2bfloat162_rn(v.z, v.w);
    }
  } else {
    const int per = width >> 1;
    for (int q = threadIdx.x; q < WG_TILE * per; q += blockDim.x) {
      const int rr = q / per, c = (q % per) * 2;
      const int64_t r = r0 + rr;
      float2 v = make_float2(0.f, 0.f);
      if (r < rend) v = *reinterpret_cast<const float2 *>(src + r * width + c);
      *reinterpret_cast<__nv_bfloat162 *>(dst + rr * ld + col0 + c) = __floats2bfloat162_rn(v.x, v.y);
    }
  }
}

__global__ void __launch_bounds__(128, 3) wgrad_kernel(int64_t n, const float *__restrict__ in0, int K0,
                                                    const float *__restrict__ in1, int K1,
                                                    const float *__restrict__ dout, float *__restrict__ part) {
  __shared__ __align__(16) __nv_bfloat16 sI[WG_TILE * WG_LDI];
  __shared__ __align__(16) __nv_bfloat16 sD[WG_TILE * WG_LDD];
  const int K = K0 + K1;
  const int KP = (K + 1 + 15) & ~15;
  const int MT = KP / 16;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q4 = lane & 3;
  const int64_t rbeg = n * blockIdx.x / gridDim.x, rend = n * (blockIdx.x + 1) / gridDim.x;
  float acc[3][8][4];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int t = 0; t < 8; t++) acc[i][t][0] = acc[i][t][1] = acc[i][t][2] = acc[i][t][3] = 0.f;
  for (int64_t r0 = rbeg; r0 < rend; r0 += WG_TILE) {
    __syncthreads();
    stage_rows(sI, WG_LDI, 0, in0, K0, r0, rend);
    if (K1 > 0) stage_rows(sI, WG_LDI, K0, in1, K1, r0, rend);
    // the ones column (bias row) and the zero padding up to KP
    for (int q = threadIdx.x; q < WG_TILE * (KP - K); q += blockDim.x) {
      const int rr = q / (KP - K), k = K + q % (KP - K);
      sI[rr * WG_LDI + k] = __float2bfloat16(k == K && r0 + rr < rend ? 1.f : 0.f);
    }
    stage_rows(sD, WG_LDD, 0, dout, 64, r0, rend);
    __syncthreads();
    const int mi = lane >> 3;
#pragma unroll
    for (int ks = 0; ks < WG_TILE / 16; ks++) {
      uint32_t bfr[8][2];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        uint32_t t[4];
        const int row = ks * 16 + (lane & 7) + (mi & 1) * 8, col = (2 * j + (mi >> 1)) * 8;
        ldsm_x4_trans(t, sD + row * WG_LDD + col);
        bfr[2 * j][0] = t[0];
        bfr[2 * j][1] = t[1];
        bfr[2 * j + 1][0] = t[2];
        bfr[2 * j + 1][1] = t[3];
      }
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const int mt = warp + 4 * i;
        if (mt >= MT) break;
        uint32_t a[4];
        const int row = ks * 16 + (lane & 7) + (mi >> 1) * 8, col = mt * 16 + (mi & 1) * 8;
        ldsm_x4_trans(a, sI + row * WG_LDI + col);
#pragma unroll
        for (int t = 0; t < 8; t++) mma_bf16(acc[i][t], a[0], a[1], a[2], a[3], bfr[t][0], bfr[t][1]);
      }
    }
  }
  // C fragment: feature rows mt*16 + g (+8), columns 8t + 2 q4 (+1)
  float *out = part + (int64_t)blockIdx.x * (K + 1) * 64;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const int mt = warp + 4 * i;
    if (mt >= MT) break;
    const int f0 = mt * 16 + g, f1 = f0 + 8;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int c = t * 8 + q4 * 2;
      if (f0 <= K) *reinterpret_cast<float2 *>(out + f0 * 64 + c) = make_float2(acc[i][t][0], acc[i][t][1]);
      if (f1 <= K) *reinterpret_cast<float2 *>(out + f1 * 64 + c) = make_float2(acc[i][t][2], acc[i][t][3]);
    }
  }
}

// grad[dst + q] (+)= sum_b part[b][q], fixed order; q < count.  The bias row
// (q >= bias_from) goes to grad[bias_dst + q - bias_from] when bias_dst >= 0.
// Blocks of 32 outputs x 8 partial groups; the groups are combined in a
// fixed order (deterministic).
__global__ void reduce_parts(int nparts, int count, const float *__restrict__ part, float *__restrict__ grad,
                             int64_t dst, int bias_from, int64_t bias_dst, int accumulate) {
  __shared__ float red[8][33];
  const int q = blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (q < count)
    for (int b = threadIdx.y; b < nparts; b += 8) s += part[(int64_t)b * count + q];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y != 0 || q >= count) return;
  s = ((red[0][threadIdx.x] + red[1][threadIdx.x]) + (red[2][threadIdx.x] + red[3][threadIdx.x])) +
      ((red[4][threadIdx.x] + red[5][threadIdx.x]) + (red[6][threadIdx.x] + red[7][threadIdx.x]));
  int64_t o;
  if (q >= bias_from) {
    if (bias_dst < 0) return;
    o = bias_dst + (q - bias_from);
  } else {
    o = dst + q;
  }
  grad[o] = accumulate ? grad[o] + s : s;
}

// g *= [r > 0] (relu mask from the post-activation)
__global__ void relu_mask(int64_t n, const float *__restrict__ r, const float *__restrict__ g,
                          float *__restrict__ out) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < n) out[q] = r[q] > 0.f ? g[q] : 0.f;
}


// Adam (Kingma & Ba 2015), bias-corrected, FP32
__global__ void adam_kernel(int64_t n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float gq = g[q];
  const float mq = b1 * m[q] + (1.f - b1) * gq, vq = b2 * v[q] + (1.f - b2) * gq * gq;
  m[q] = mq;
  v[q] = vq;
  p[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
}

// ----------------------------------------------------------- features
// unit phase factor k (normalized in place by normalize_phases)
__device__ __forceinline__ void phases(const double *c, int k, double &er, double &ei) {
  er = c[2 * k];
  ei = c[2 * k + 1];
}

// per node: s = x0 - x1, q = quad - sec, c = cubic - quad at t (fields in
// sq, 6 doubles per node), the sums of |s|^2, |q|^2, |c|^2 into red[0..2],
// and (when sec_out is given) the secant prediction itself
__global__ void features_a(int64_t n, const double *__restrict__ dots, const double *__restrict__ Ls,
                           const C2<double> *__restrict__ x0, const C2<double> *__restrict__ x1,
                           const C2<double> *__restrict__ x2, const C2<double> *__restrict__ x3,
                           double *__restrict__ sq, C2<double> *__restrict__ sec_out, double *partials,
                           unsigned *counter, double *red) {
  double er[3], ei[3];
  for (int k = 0; k < 3; k++) phases(dots, k, er[k], ei[k]);
  double as = 0.0, aq = 0.0, ac = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double xr[4], xi[4];
    xr[0] = x0[i].x;
    xi[0] = x0[i].y;
    const C2<double> *xs[3] = {x1, x2, x3};
    for (int k = 0; k < 3; k++) {
      const C2<double> p = xs[k][i];
      xr[k + 1] = er[k] * p.x - ei[k] * p.y;
      xi[k + 1] = er[k] * p.y + ei[k] * p.x;
    }
    // Ls: secant (2), quadratic (3), cubic (4) Lagrange weights
    const double secr = Ls[0] * xr[0] + Ls[1] * xr[1], seci = Ls[0] * xi[0] + Ls[1] * xi[1];
    const double qdr = Ls[2] * xr[0] + Ls[3] * xr[1] + Ls[4] * xr[2];
    const double qdi = Ls[2] * xi[0] + Ls[3] * xi[1] + Ls[4] * xi[2];
    const double cbr = Ls[5] * xr[0] + Ls[6] * xr[1] + Ls[7] * xr[2] + Ls[8] * xr[3];
    const double cbi = Ls[5] * xi[0] + Ls[6] * xi[1] + Ls[7] * xi[2] + Ls[8] * xi[3];
    if (sec_out) sec_out[i] = C2<double>{secr, seci};
    double *o = sq + 6 * i;
    o[0] = xr[0] - xr[1];
    o[1] = xi[0] - xi[1];
    o[2] = qdr - secr;
    o[3] = qdi - seci;
    o[4] = cbr - qdr;
    o[5] = cbi - qdi;
    as += o[0] * o[0] + o[1] * o[1];
    aq += o[2] * o[2] + o[3] * o[3];
    ac += o[4] * o[4] + o[5] * o[5];
  }
  const double v[3] = {as, aq, ac};
  grid_reduce_n<3>(v, 3, partials, counter, red);
}

// X = [x0, s~, q~, c~, mu_new, 1]
__global__ void features_b(int64_t n, const double *__restrict__ red, double mu_new,
                           const C2<double> *__restrict__ x0, const double *__restrict__ sq,
                           float *__restrict__ X) {
  // the inverse RMS scales in FP32 (the features are FP32): an FP64 square
  // root and division per thread cost more than the whole pass
  const float fn = (float)n;
  const float rs = sqrtf((float)red[0] / fn), rq = sqrtf((float)red[1] / fn), rc = sqrtf((float)red[2] / fn);
  const double is = rs > 0.f ? (double)(1.f / rs) : 0.0, iq = rq > 0.f ? (double)(1.f / rq) : 0.0,
               ic = rc > 0.f ? (double)(1.f / rc) : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const C2<double> a = x0[i];
    const double *f = sq + 6 * i;
    float *xi = X + i * FX;
    xi[0] = (float)a.x;
    xi[1] = (float)a.y;
    xi[2] = (float)(f[0] * is);
    xi[3] = (float)(f[1] * is);
    xi[4] = (float)(f[2] * iq);
    xi[5] = (float)(f[3] * iq);
    xi[6] = (float)(f[4] * ic);
    xi[7] = (float)(f[5] * ic);
    xi[8] = (float)mu_new;
    xi[9] = 1.f;
  }
}

// The training sample's error fields: c (cubic - quadratic), d = e_t x_t -
// quadratic (the quadratic prediction's error) and the phase-aligned target
// e_t x_t, as complex vectors.
__global__ void sample_fields(int64_t n, const double *__restrict__ dots, const double *__restrict__ Ls,
                              const C2<double> *__restrict__ x0, const C2<double> *__restrict__ x1,
                              const C2<double> *__restrict__ xt, const double *__restrict__ sq,
                              C2<double> *__restrict__ c_out, C2<double> *__restrict__ d_out,
                              C2<double> *__restrict__ t_out) {
  double e1r, e1i, etr, eti;
  phases(dots, 0, e1r, e1i);
  phases(dots, 3, etr, eti);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const C2<double> a = x0[i], p = x1[i], t = xt[i];
    const double pr = e1r * p.x - e1i * p.y, pi = e1r * p.y + e1i * p.x;
    const double *f = sq + 6 * i;
    const double qr = Ls[0] * a.x + Ls[1] * pr + f[2], qi = Ls[0] * a.y + Ls[1] * pi + f[3];
    const double tr = etr * t.x - eti * t.y, ti = etr * t.y + eti * t.x;
    c_out[i] = C2<double>{f[4], f[5]};
    d_out[i] = C2<double>{tr - qr, ti - qi};
    t_out[i] = C2<double>{tr, ti};
  }
}

// g = [<u,u>, <u,v>, <v,v>] over 2n reals
__global__ void gram3_kernel(int64_t n2, const double *__restrict__ u, const double *__restrict__ v,
                             double *partials, unsigned *counter, double *g) {
  double acc[3] = {0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
    const double a = u[i], b = v[i];
    acc[0] += a * a;
    acc[1] += a * b;
    acc[2] += b * b;
  }
  grid_reduce_n<3>(acc, 3, partials, counter, g);
}

// features_a's prediction fields and combine_kernel's sum in one pass, with
// the same operations in the same order (bitwise the two-kernel result):
// the secant into sec_out, out = sec + (q + w c)
__global__ void predict_fields_kernel(int64_t n, const double *__restrict__ dots, const double *__restrict__ Ls,
                                      const double *__restrict__ w, const C2<double> *__restrict__ x0,
                                      const C2<double> *__restrict__ x1, const C2<double> *__restrict__ x2,
                                      const C2<double> *__restrict__ x3, C2<double> *__restrict__ sec_out,
                                      C2<double> *__restrict__ out) {
  double er[3], ei[3];
  for (int k = 0; k < 3; k++) phases(dots, k, er[k], ei[k]);
  const double wc = w[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double xr[4], xi[4];
    xr[0] = x0[i].x;
    xi[0] = x0[i].y;
    const C2<double> *xs[3] = {x1, x2, x3};
    for (int k = 0; k < 3; k++) {
      const C2<double> p = xs[k][i];
      xr[k + 1] = er[k] * p.x - ei[k] * p.y;
      xi[k + 1] = er[k] * p.y + ei[k] * p.x;
    }
    const double secr = Ls[0] * xr[0] + Ls[1] * xr[1], seci = Ls[0] * xi[0] + Ls[1] * xi[1];
    const double qdr = Ls[2] * xr[0] + Ls[3] * xr[1] + Ls[4] * xr[2];
    const double qdi = Ls[2] * xi[0] + Ls[3] * xi[1] + Ls[4] * xi[2];
    const double cbr = Ls[5] * xr[0] + Ls[6] * xr[1] + Ls[7] * xr[2] + Ls[8] * xr[3];
    const double cbi = Ls[5] * xi[0] + Ls[6] * xi[1] + Ls[7] * xi[2] + Ls[8] * xi[3];
    sec_out[i] = C2<double>{secr, seci};
    const double f2 = qdr - secr, f3 = qdi - seci, f4 = cbr - qdr, f5 = cbi - qdi;
    C2<double> o{secr, seci};
    o.x += f2 + wc * f4;
    o.y += f3 + wc * f5;
    out[i] = o;
  }
}

// out = sec + q + w c (sec: the secant prediction)
__global__ void combine_kernel(int64_t n, const double *__restrict__ w, const double *__restrict__ sq,
                               const C2<double> *__restrict__ sec, C2<double> *__restrict__ out) {
  const double wc = w[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double *f = sq + 6 * i;
    C2<double> o = sec[i];
    o.x += f[2] + wc * f[4];
    o.y += f[3] + wc * f[5];
    out[i] = o;
  }
}

// ------------------------------------------------------------- readout
// z = sum of the pool partials / n; w = relu(z W1 + b1) W2 + b2.  With a
// Gram vector [cc, cd, dd]: the loss (w^2 cc - 2 w cd + dd) / dd, the
// backward pass of the readout into grad and dz.  One CTA of 256 threads.
__global__ void readout(int nparts, int64_t n, const float *__restrict__ part, const float *__restrict__ P,
                        int64_t o_w1, int64_t o_b1, int64_t o_w2, int64_t o_b2, double *__restrict__ wout,
                        const double *__restrict__ gram, float *__restrict__ grad, float *__restrict__ dz,
                        double *__restrict__ loss) {
  __shared__ float z[H], zs[4][H], h1[RH], dh1[RH];
  __shared__ double dw;
  const int t = threadIdx.x;
  {
    const int c = t & (H - 1), grp = t / H;  // 4 groups of 64 channels
    float a0 = 0.f, a1 = 0.f;
    int b = grp;
    for (; b + 4 < nparts; b += 8) {
      a0 += part[(int64_t)b * H + c];
      a1 += part[(int64_t)(b + 4) * H + c];
    }
    for (; b < nparts; b += 4) a0 += part[(int64_t)b * H + c];
    zs[grp][c] = a0 + a1;
  }
  __syncthreads();
  if (t < H) z[t] = ((zs[0][t] + zs[1][t]) + (zs[2][t] + zs[3][t])) / (float)n;
  __syncthreads();
  if (t < RH) {
    float a = P[o_b1 + t];
    for (int k = 0; k < H; k++) a += z[k] * P[o_w1 + k * RH + t];
    h1[t] = fmaxf(a, 0.f);
  }
  __syncthreads();
  if (t == 0) {
    double a = P[o_b2];
    for (int k = 0; k < RH; k++) a += (double)h1[k] * P[o_w2 + k];
    *wout = a;
    if (gram) {
      const double dd = gram[2] > 0 ? gram[2] : 1.0;
      *loss = (a * a * gram[0] - 2 * a * gram[1] + gram[2]) / dd;
      dw = 2 * (a * gram[0] - gram[1]) / dd;
    }
  }
  __syncthreads();
  if (!gram) return;
  if (t < RH) {
    // W2, b2 gradients and dh1
    grad[o_w2 + t] = (float)(h1[t] * dw);
    const float g = (float)(dw * P[o_w2 + t]);
    dh1[t] = h1[t] > 0.f ? g : 0.f;
  }
  if (t == 0) grad[o_b2] = (float)dw;
  __syncthreads();
  // W1, b1 gradients and dz
  for (int q = t; q < H * RH; q += blockDim.x) grad[o_w1 + q] = z[q / RH] * dh1[q % RH];
  if (t < RH) grad[o_b1 + t] = dh1[t];
  if (t < H) {
    float a = 0.f;
    for (int k = 0; k < RH; k++) a += dh1[k] * P[o_w1 + t * RH + k];
    dz[t] = a;
  }
}

// dh[i][c] = dz[c] / n (gradient of the mean pool)
__global__ void pool_backward(int64_t n, const float *__restrict__ dz, float *__restrict__ dh) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < n * H) dh[q] = dz[q % H] / (float)n;
}


// per-nonzero edge features and the transpose map of the symmetric graph
__global__ void edge_setup(int64_t nnz, const int32_t *__restrict__ nz_edge, const int32_t *__restrict__ pf,
                           const int32_t *__restrict__ pb, const double *__restrict__ alpha,
                           const double *__restrict__ p, const double *__restrict__ len, double ia, double ip,
                           double il, float *__restrict__ ef, int32_t *__restrict__ tr) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const int32_t z = nz_edge[k];
  const int32_t e = z >= 0 ? z : ~z;
  const double sgn = z >= 0 ? 1.0 : -1.0;
  float4 f;
  f.x = (float)(alpha[e] * ia);
  f.y = (float)(sgn * p[e] * ip);
  f.z = (float)(len[e] * il);
  f.w = 1.f;
  *reinterpret_cast<float4 *>(ef + k * FE) = f;
  tr[k] = z >= 0 ? pb[e] : pf[e];
}

inline int vgrid(int64_t n) { return (int)std::min<int64_t>(div_up(n, 256), kNumSMs * 8); }

// resident CTAs of a 128-thread kernel on the whole device, capped by the
// number of tiles
int persistent_grid(const void *kernel, size_t smem, int64_t tiles) {
  int d = 0, sms = 0, per_sm = 0;
  NOSH_CUDA(cudaGetDevice(&d));
  NOSH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d));
  NOSH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, smem));
  return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)std::max(per_sm, 1) * sms));
}

// splitmix64 for deterministic initialisation
inline uint64_t sm64(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

}  // namespace

// ------------------------------------------------------------------ impl
struct Mpnn::Impl {
  NlsImpl &s;
  Layout L;
  int64_t N, nnz;
  DevBuf<float> ef;
  DevBuf<int32_t> tr;
  DevBuf<float> params, grads, am, av;
  int64_t adam_t = 0;
  // BF16 transposed operands: forward W (enc padded to K=16, wa, wb, wu per
  // layer) and the W^T blocks of the backward pass
  DevBuf<__nv_bfloat16> wt;
  int64_t wt_enc, wt_a[LAYERS], wt_b[LAYERS], wt_u[LAYERS], wtb_a[LAYERS], wtb_b[LAYERS], wtb_uh[LAYERS],
      wtb_um[LAYERS];
  // activations (A, B in FP16: the message operands) and gradients
  DevBuf<float> X, Hs[LAYERS], Mg[LAYERS], R[LAYERS];
  DevBuf<__half> A[LAYERS], B[LAYERS];
  DevBuf<float> dH, dR, dM, dA, dB, dz;
  DevBuf<float> part, pool;
  DevBuf<__nv_bfloat16> Mb;  // inference split: one layer's M in BF16
  int enc_grid = 0, layer_grid = 0, agg_grid = 0, upd_grid = 0;
  int pool_parts = 0;  // pool partial rows written by the last forward
  DevBuf<double> sq, red, dots, Ls, gram, w, loss;
  DevBuf<double> vc, vd, vt, jc, jd;  // training sample fields and their J applies
  // launches go to `stream`: the handle's stream, or a side stream while an
  // inference overlaps the solver; own reduction scratch for the features
  cudaStream_t stream;
  Reducer rd;
  explicit Impl(NlsImpl &nls);
  void refresh_bf16();
  void forward(bool train);               // X -> pooled embedding
  double backward_and_step(float lr);     // needs gram
  void features(const double *const x[4], const double mu[4], double mu_t, const double *target,
                double *secant = nullptr, bool node_features = true);
  // Lagrange weights (into Ls) and phase factors of x[1..3] (and target)
  // against x[0] (into dots)
  void align(const double *const x[4], const double mu[4], double t, const double *target);
  void gemm(int epi, const float *in0, int K0, const float *in1, int K1, int64_t wt_off, float *out);
  void wgrad(const float *in0, int K0, const float *in1, int K1, const float *dout, int ncol, int64_t dst,
             int64_t bias_dst);
  void readout_launch(bool train);
};

Mpnn::Impl::Impl(NlsImpl &nls) : s(nls), N(nls.N), nnz(2 * nls.E), stream(nls.stream) {
  cudaStream_t st = s.stream;
  rd.init(2 * (vgrid(N) + 64), 4, st);  // history_dots: up to 8 slots of partials
  MeshImpl &m = *s.mesh;
  // normalisation of the edge features from the mesh and fields
  std::vector<double> alpha(s.E), p(s.E);
  s.d_alpha.download(alpha.data(), s.E, st);
  s.d_p.download(p.data(), s.E, st);
  s.sync();
  double sa = 0, sp = 0, sl = 0;
  for (int64_t e = 0; e < s.E; e++) {
    sa += std::fabs(alpha[e]);
    sp += p[e] * p[e];
    sl += m.h_len[e];
  }
  const double ia = sa > 0 ? s.E / sa : 1.0, ip = sp > 0 ? 1.0 / std::sqrt(sp / s.E) : 1.0,
               il = sl > 0 ? s.E / sl : 1.0;
  ef.alloc(nnz * FE);
  tr.alloc(nnz);
  edge_setup<<<div_up(nnz, 256), 256, 0, st>>>(nnz, m.d_nz_edge.p, m.d_pos_fwd.p, m.d_pos_bwd.p, s.d_alpha.p,
                                               s.d_p.p, m.d_len.p, ia, ip, il, ef.p, tr.p);
  NOSH_CUDA(cudaGetLastError());
  // parameters: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero
  // biases; the readout starts near w = (1, 1), the cubic extrapolation
  // (the Lagrange combination of the four states), with small weights
  std::vector<float> h(L.total, 0.f);
  uint64_t seed = 0x6e6f7368ULL;
  auto fill = [&](int64_t off, int64_t count, int fan_in, float scale) {
    const float b = scale / std::sqrt((float)fan_in);
    for (int64_t q = 0; q < count; q++) h[off + q] = b * (2.f * (float)((sm64(seed) >> 11) * 0x1.0p-53) - 1.f);
  };
  fill(L.enc_w, FX * H, FX, 1.f);
  for (int l = 0; l < LAYERS; l++) {
    fill(L.wa[l], H * H, H, 1.f);
    fill(L.wb[l], H * H, H, 1.f);
    fill(L.wc[l], FE * H, FE, 1.f);
    fill(L.wu[l], 2 * H * H, 2 * H, 1.f);
  }
  fill(L.r1_w, H * RH, H, 1.f);
  fill(L.r2_w, RH, RH, 0.01f);
  h[L.r2_b] = 1.f;
  params.upload(h, st);
  grads.alloc(L.total);
  grads.zero(st);
  am.alloc(L.total);
  av.alloc(L.total);
  am.zero(st);
  av.zero(st);
  int64_t o = 0;
  wt_enc = o; o += H * 16;
  for (int l = 0; l < LAYERS; l++) {
    wt_a[l] = o; o += H * H;
    wt_b[l] = o; o += H * H;
    wt_u[l] = o; o += H * 2 * H;
    wtb_a[l] = o; o += H * H;
    wtb_b[l] = o; o += H * H;
    wtb_uh[l] = o; o += H * H;
    wtb_um[l] = o; o += H * H;
  }
  wt.alloc(o);
  wt.zero(st);
  X.alloc(N * FX);
  for (int l = 0; l < LAYERS; l++) {
    Hs[l].alloc(N * H);
    A[l].alloc(N * H);
    B[l].alloc(N * H);
    Mg[l].alloc(N * H);
    R[l].alloc(N * H);
  }
  for (DevBuf<float> *b : {&dH, &dR, &dM, &dA, &dB}) b->alloc(N * H);
  dz.alloc(H);
  part.alloc(std::max<int64_t>((int64_t)WG_PARTS * (2 * H + 1) * H, div_up(N, 64) * 5 * H) + 64);
  const int64_t tiles = div_up(N, (int64_t)TILE);
  enc_grid = persistent_grid((const void *)encode_kernel, kEncSmem, tiles);
  layer_grid = persistent_grid((const void *)mp_layer_kernel<true, true, false>, kLayerSmem, tiles);
  for (const void *k : {(const void *)mp_layer_kernel<false, false, false>,
                        (const void *)mp_layer_kernel<false, true, false>,
                        (const void *)mp_layer_kernel<true, false, false>})
    layer_grid = std::min(layer_grid, persistent_grid(k, kLayerSmem, tiles));
  upd_grid = std::min(persistent_grid((const void *)mp_layer_kernel<false, false, true>, kUpdateSmem, tiles),
                      persistent_grid((const void *)mp_layer_kernel<false, true, true>, kUpdateSmem, tiles));
  {
    int d = 0, sms = 0, per_sm = 0;
    NOSH_CUDA(cudaGetDevice(&d));
    NOSH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d));
    NOSH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mp_aggregate_kernel, 256, 0));
    // 16 rows per CTA pass (8 warps, a half-warp per row)
    agg_grid = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(N, 16), (int64_t)std::max(per_sm, 1) * sms));
  }
  Mb.alloc(N * H);
  pool.alloc((int64_t)std::max(layer_grid, upd_grid) * H);
  sq.alloc(6 * N);
  red.alloc(8);
  dots.alloc(8);
  Ls.alloc(9);
  gram.alloc(3);
  w.alloc(1);
  w.zero(st);
  loss.alloc(1);
  refresh_bf16();
  s.sync();
}

void Mpnn::Impl::refresh_bf16() {
  cudaStream_t st = stream;
  const float *P = params.p;
  // encoder: K = 10 features padded to 16 (zero weights in the padding)
  enc_to_bf16<<<div_up(H * 16, 256), 256, 0, st>>>(P + L.enc_w, wt.p + wt_enc);
  for (int l = 0; l < LAYERS; l++) {
    to_bf16_t<<<div_up(H * H, 256), 256, 0, st>>>(P + L.wa[l], H, H, 0, wt.p + wt_a[l]);
    to_bf16_t<<<div_up(H * H, 256), 256, 0, st>>>(P + L.wb[l], H, H, 0, wt.p + wt_b[l]);
    to_bf16_t<<<div_up(H * 2 * H, 256), 256, 0, st>>>(P + L.wu[l], 2 * H, H, 0, wt.p + wt_u[l]);
    // backward operands: dIn = dOut W^T  ->  Wt[n][k] = W[n][k]
    to_bf16_rows<<<div_up(H * H, 256), 256, 0, st>>>(P + L.wa[l], H, 0, wt.p + wtb_a[l]);
    to_bf16_rows<<<div_up(H * H, 256), 256, 0, st>>>(P + L.wb[l], H, 0, wt.p + wtb_b[l]);
    to_bf16_rows<<<div_up(H * H, 256), 256, 0, st>>>(P + L.wu[l], 2 * H, 0, wt.p + wtb_uh[l]);
    to_bf16_rows<<<div_up(H * H, 256), 256, 0, st>>>(P + L.wu[l], 2 * H, H, wt.p + wtb_um[l]);
  }
  s.launch_count += 1 + 7 * LAYERS;
  NOSH_CUDA(cudaGetLastError());
}

void Mpnn::Impl::gemm(int epi, const float *in0, int K0, const float *in1, int K1, int64_t wt_off, float *out) {
  const int grid = div_up(N, 64);
  cudaStream_t st = stream;
  const __nv_bfloat16 *W = wt.p + wt_off;
  switch (epi) {
    case EPI_LINEAR: gemm64_kernel<EPI_LINEAR><<<grid, 128, 0, st>>>(N, in0, K0, in1, K1, W, out); break;
    default: gemm64_kernel<EPI_ACCUM><<<grid, 128, 0, st>>>(N, in0, K0, in1, K1, W, out); break;
  }
  ++s.launch_count;
}

void Mpnn::Impl::readout_launch(bool train) {
  cudaStream_t st = stream;
  readout<<<1, 4 * H, 0, st>>>(pool_parts, N, pool.p, params.p, L.r1_w, L.r1_b, L.r2_w, L.r2_b, w.p,
                               train ? gram.p : nullptr, grads.p, dz.p, loss.p);
  ++s.launch_count;
}

void Mpnn::Impl::forward(bool train) {
  cudaStream_t st = stream;
  const float *P = params.p;
  MeshImpl &m = *s.mesh;
  const float4 *ef4 = reinterpret_cast<const float4 *>(ef.p);
  encode_kernel<<<enc_grid, 128, kEncSmem, st>>>(N, X.p, wt.p + wt_enc, P + L.enc_b, wt.p + wt_a[0], Hs[0].p,
                                                 A[0].p, B[0].p);
  ++s.launch_count;
  for (int l = 0; l < LAYERS; l++) {
    const bool last = l == LAYERS - 1;
    if (train) {
      // fused layer (it also stores M and R for the backward pass)
      auto kernel = last ? mp_layer_kernel<true, true, false> : mp_layer_kernel<true, false, false>;
      kernel<<<layer_grid, 128, kLayerSmem, st>>>(
          N, m.d_rp.p, m.d_ci.p, ef4, Hs[l].p, A[l].p, B[l].p, P + L.wc[l], P + L.bm[l], wt.p + wt_u[l],
          P + L.bu[l], last ? nullptr : wt.p + wt_a[l + 1], last ? nullptr : Hs[l + 1].p,
          last ? nullptr : A[l + 1].p, last ? nullptr : B[l + 1].p, Mg[l].p, R[l].p, pool.p, nullptr);
      pool_parts = layer_grid;
    } else {
      // inference: the aggregation at high occupancy, then the update GEMM
      // (bitwise the fused layer's result: the same arithmetic and the
      // same BF16 rounding of M)
      mp_aggregate_kernel<<<agg_grid, 256, 0, st>>>(N, m.d_rp.p, m.d_ci.p, ef4, A[l].p, B[l].p, P + L.wc[l],
                                                    P + L.bm[l], Mb.p);
      auto kernel = last ? mp_layer_kernel<false, true, true> : mp_layer_kernel<false, false, true>;
      kernel<<<upd_grid, 128, kUpdateSmem, st>>>(
          N, m.d_rp.p, m.d_ci.p, ef4, Hs[l].p, A[l].p, B[l].p, P + L.wc[l], P + L.bm[l], wt.p + wt_u[l],
          P + L.bu[l], last ? nullptr : wt.p + wt_a[l + 1], last ? nullptr : Hs[l + 1].p,
          last ? nullptr : A[l + 1].p, last ? nullptr : B[l + 1].p, nullptr, nullptr, pool.p, Mb.p);
      pool_parts = upd_grid;
      ++s.launch_count;
    }
    ++s.launch_count;
  }
  NOSH_CUDA(cudaGetLastError());
}

void Mpnn::Impl::wgrad(const float *in0, int K0, const float *in1, int K1, const float *dout, int ncol,
                       int64_t dst, int64_t bias_dst) {
  cudaStream_t st = stream;
  (void)ncol;  // always H
  const int nb = (int)std::min<int64_t>(WG_PARTS, std::max<int64_t>(1, div_up(N, 4 * WG_TILE)));
  const int count = (K0 + K1 + 1) * H;
  wgrad_kernel<<<nb, 128, 0, st>>>(N, in0, K0, in1, K1, dout, part.p);
  reduce_parts<<<div_up(count, 32), dim3(32, 8), 0, st>>>(nb, count, part.p, grads.p, dst, (K0 + K1) * H, bias_dst,
                                                          0);
  s.launch_count += 2;
}

// forward must have run; gram holds the sample's Gram scalars
double Mpnn::Impl::backward_and_step(float lr) {
  cudaStream_t st = stream;
  const float *P = params.p;
  MeshImpl &m = *s.mesh;
  readout_launch(true);  // loss, readout gradients, dz
  pool_backward<<<div_up(N * H, 256), 256, 0, st>>>(N, dz.p, dH.p);
  ++s.launch_count;
  for (int l = LAYERS - 1; l >= 0; l--) {
    // h_{l+1} = h_l + R_l, R_l = relu([h_l, M_l] W_u + b_u)
    relu_mask<<<div_up(N * H, 256), 256, 0, st>>>(N * H, R[l].p, dH.p, dR.p);
    ++s.launch_count;
    wgrad(Hs[l].p, H, Mg[l].p, H, dR.p, H, L.wu[l], L.bu[l]);
    // dM = dR W_u[64:128]^T ; dh += dR W_u[0:64]^T (dh holds the residual path)
    gemm(EPI_LINEAR, dR.p, H, nullptr, 0, wtb_um[l], dM.p);
    gemm(EPI_ACCUM, dR.p, H, nullptr, 0, wtb_uh[l], dH.p);
    const int nb = div_up(N, EB_ROWS);
    const float4 *ef4 = reinterpret_cast<const float4 *>(ef.p);
    edge_backward_a<<<nb, 256, 0, st>>>(N, m.d_rp.p, m.d_ci.p, ef4, A[l].p, B[l].p, P + L.wc[l], P + L.bm[l],
                                        dM.p, dA.p, part.p);
    reduce_parts<<<div_up(5 * H, 32), dim3(32, 8), 0, st>>>(nb, 5 * H, part.p, grads.p, L.wc[l], 4 * H, L.bm[l],
                                                             0);
    edge_backward_b<<<nb, 256, 0, st>>>(N, m.d_rp.p, m.d_ci.p, tr.p, ef4, A[l].p, B[l].p, P + L.wc[l],
                                        P + L.bm[l], dM.p, dB.p);
    s.launch_count += 3;
    // A = h W_a, B = h W_b
    wgrad(Hs[l].p, H, nullptr, 0, dA.p, H, L.wa[l], -1);
    wgrad(Hs[l].p, H, nullptr, 0, dB.p, H, L.wb[l], -1);
    gemm(EPI_ACCUM, dA.p, H, nullptr, 0, wtb_a[l], dH.p);
    gemm(EPI_ACCUM, dB.p, H, nullptr, 0, wtb_b[l], dH.p);
  }
  // encoder: h0 = relu(X W + b)
  relu_mask<<<div_up(N * H, 256), 256, 0, st>>>(N * H, Hs[0].p, dH.p, dR.p);
  ++s.launch_count;
  wgrad(X.p, FX, nullptr, 0, dR.p, H, L.enc_w, L.enc_b);
  if (lr > 0.f) {
    adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
    adam_kernel<<<div_up(L.total, 256), 256, 0, st>>>(L.total, params.p, grads.p, am.p, av.p, lr, b1, b2, 1e-8f,
                                                      c1, c2);
    ++s.launch_count;
    refresh_bf16();
  }
  double hl = 0.0;
  loss.download(&hl, 1, st);
  NOSH_CUDA(cudaStreamSynchronize(st));
  return hl;
}

// node features at mu_t from the newest states x[0..3] (mu[0..3]) and, with
// a target (the converged state at mu_t), the sample's Gram scalars
void Mpnn::Impl::align(const double *const x[4], const double mu[4], double t, const double *target) {
  cudaStream_t st = stream;
  double Lh[9];
  Lh[0] = (t - mu[1]) / (mu[0] - mu[1]);
  Lh[1] = (t - mu[0]) / (mu[1] - mu[0]);
  for (int k = 0; k < 3; k++) {
    double v = 1.0;
    for (int q = 0; q < 3; q++)
      if (q != k) v *= (t - mu[q]) / (mu[k] - mu[q]);
    Lh[2 + k] = v;
  }
  for (int k = 0; k < 4; k++) {
    double v = 1.0;
    for (int q = 0; q < 4; q++)
      if (q != k) v *= (t - mu[q]) / (mu[k] - mu[q]);
    Lh[5 + k] = v;
  }
  Ls.upload(Lh, 9, st);
  // <x_k, x_0> for x_1..x_3 and the target, x_0 read once
  history_dots<<<reduce_grid(N), 256, 0, st>>>(N, x[0], x[1], x[2], x[3], target, target ? 4 : 3, rd.partials.p,
                                  rd.counter.p, dots.p);
  ++s.launch_count;
  normalize_phases<<<1, 32, 0, st>>>(target ? 4 : 3, dots.p);
  ++s.launch_count;
}

void Mpnn::Impl::features(const double *const x[4], const double mu[4], double t, const double *target,
                          double *secant, bool node_features) {
  cudaStream_t st = stream;
  const int G = vgrid(N);
  align(x, mu, t, target);
  features_a<<<reduce_grid(N), 256, 0, st>>>(N, dots.p, Ls.p, (const C2<double> *)x[0], (const C2<double> *)x[1],
                                (const C2<double> *)x[2], (const C2<double> *)x[3], sq.p, (C2<double> *)secant,
                                rd.partials.p,
                                rd.counter.p, red.p);
  ++s.launch_count;
  if (node_features || target) {  // the network's input (not needed by combine alone)
    features_b<<<G, 256, 0, st>>>(N, red.p, t, (const C2<double> *)x[0], sq.p, X.p);
    ++s.launch_count;
  }
  if (target) {
    // The loss is the linearised residual of the prediction, relative to
    // the quadratic's: F(q + w c) ~ J (w c - d) with J at the aligned target
    // (F there is ~0), so g = [|Jc|^2, <Jc, Jd>, |Jd|^2].  The residual is
    // what Newton starts from; a state-space (cv-weighted) error favoured
    // the cubic combination, whose amplified high-frequency noise the
    // residual penalises.
    if (vc.n < (size_t)(2 * N))
      for (DevBuf<double> *b : {&vc, &vd, &vt, &jc, &jd}) b->alloc(2 * N);
    sample_fields<<<G, 256, 0, st>>>(N, dots.p, Ls.p, (const C2<double> *)x[0], (const C2<double> *)x[1],
                                     (const C2<double> *)target, sq.p, (C2<double> *)vc.p, (C2<double> *)vd.p,
                                     (C2<double> *)vt.p);
    ++s.launch_count;
    s.jac_rebuild(vt.p, s.g0, t);
    s.jac_apply<double>(vc.p, jc.p);
    s.jac_apply<double>(vd.p, jd.p);
    gram3_kernel<<<reduce_grid(2 * N), 256, 0, st>>>(2 * N, jc.p, jd.p, rd.partials.p, rd.counter.p, gram.p);
    s.launch_count += 3;
  }
  NOSH_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------- facade
Mpnn::Mpnn(NlsImpl &s) : impl(new Impl(s)) {}
Mpnn::~Mpnn() = default;

double Mpnn::predict(const double *const x[4], const double mu[4], double mu_new, double *secant, double *out) {
  Impl &I = *impl;
  I.features(x, mu, mu_new, nullptr, secant);
  I.forward(false);
  I.readout_launch(false);
  combine_kernel<<<vgrid(I.N), 256, 0, I.s.stream>>>(I.N, I.w.p, I.sq.p, (const C2<double> *)secant,
                                                     (C2<double> *)out);
  ++I.s.launch_count;
  NOSH_CUDA(cudaGetLastError());
  double w = 0.0;
  I.w.download(&w, 1, I.s.stream);  // pageable destination: returns once copied
  return w;
}

void Mpnn::prepare(const double *const x[4], const double mu[4], double mu_new, double *secant,
                   bool node_features) {
  impl->features(x, mu, mu_new, nullptr, secant, node_features);
}

void Mpnn::infer(cudaStream_t st) {
  Impl &I = *impl;
  I.stream = st;
  I.forward(false);
  I.readout_launch(false);
  I.stream = I.s.stream;
}

void Mpnn::combine(const double *secant, double *out, double *w_host) {
  Impl &I = *impl;
  combine_kernel<<<vgrid(I.N), 256, 0, I.s.stream>>>(I.N, I.w.p, I.sq.p, (const C2<double> *)secant,
                                                     (C2<double> *)out);
  ++I.s.launch_count;
  NOSH_CUDA(cudaGetLastError());
  if (w_host) NOSH_CUDA(cudaMemcpyAsync(w_host, I.w.p, sizeof(double), cudaMemcpyDeviceToHost, I.s.stream));
}

void Mpnn::predict_fields(const double *const x[4], const double mu[4], double mu_new, double *secant, double *out,
                          double *w_host) {
  Impl &I = *impl;
  I.align(x, mu, mu_new, nullptr);
  predict_fields_kernel<<<vgrid(I.N), 256, 0, I.s.stream>>>(
      I.N, I.dots.p, I.Ls.p, I.w.p, (const C2<double> *)x[0], (const C2<double> *)x[1], (const C2<double> *)x[2],
      (const C2<double> *)x[3], (C2<double> *)secant, (C2<double> *)out);
  ++I.s.launch_count;
  NOSH_CUDA(cudaGetLastError());
  if (w_host) NOSH_CUDA(cudaMemcpyAsync(w_host, I.w.p, sizeof(double), cudaMemcpyDeviceToHost, I.s.stream));
}

double Mpnn::train(const double *const x[4], const double mu[4], const double *target, double mu_t, int iters,
                   double lr) {
  Impl &I = *impl;
  I.features(x, mu, mu_t, target);
  double l = std::nan("");
  for (int k = 0; k < iters; k++) {
    I.forward(true);
    l = I.backward_and_step((float)lr);
  }
  return l;
}

// ------------------------------------------ hooks for the gradient checks
int64_t Mpnn::num_params() const { return impl->L.total; }
void Mpnn::get_params(float *h) const {
  impl->params.download(h, impl->L.total, impl->s.stream);
  impl->s.sync();
}
void Mpnn::set_params(const float *h) {
  impl->params.upload(h, impl->L.total, impl->s.stream);
  impl->refresh_bf16();
  impl->s.sync();
}
void Mpnn::get_edge_features(float *h) const {
  impl->ef.download(h, impl->nnz * FE, impl->s.stream);
  impl->s.sync();
}
void Mpnn::forward_features(const float *X, double *w) {
  Impl &I = *impl;
  I.X.upload(X, I.N * FX, I.s.stream);
  I.forward(false);
  I.readout_launch(false);
  I.w.download(w, 1, I.s.stream);
  I.s.sync();
}
double Mpnn::loss_and_grad(const float *X, const double *gram, float *grad) {
  Impl &I = *impl;
  I.X.upload(X, I.N * FX, I.s.stream);
  I.gram.upload(gram, 3, I.s.stream);
  I.forward(true);
  const double l = I.backward_and_step(0.f);  // gradient only, no step
  I.grads.download(grad, I.L.total, I.s.stream);
  I.s.sync();
  return l;
}

}  // namespace nosh
