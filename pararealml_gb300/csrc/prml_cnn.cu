/*
 * Residual CNN coarse propagator: forward, backward and optimiser kernels.
 *
 * Network (for a 2-component state u on an H x W grid):
 *   x1 = relu(conv3x3(s_in * u; w0 [9][2][32]) + b0)          CUDA cores
 *   x{l+1} = relu(conv3x3(x_l; w_l [9][32][32]) + b_l), l=1..4  tensor cores
 *   y  = u + s_out * (conv3x3(x5; w5 [9][32][2]) + b5)         CUDA cores
 * "same" convolutions with zero padding; taps ordered t = (dy+1)*3 + (dx+1).
 *
 * Hidden activations and their gradients are bfloat16 NHWC [B][H][W][32];
 * the 32 -> 32 convolutions are implicit GEMMs on the tensor cores
 * (ldmatrix + mma.sync m16n8k16, bf16 x bf16 -> fp32): M = pixels,
 * N = output channels, K = 9 taps x 32 input channels.  The tap shift is a
 * per-row shared-memory address, so the 3x3 halo patch of a tile is staged
 * once (cp.async, zero fill outside the image) and reused by all 9 taps.
 *
 * Backward: dgrad of a 32 -> 32 layer is the same kernel with the weights
 * transposed and the taps flipped, and the ReLU mask of the layer input in
 * place of bias + ReLU; wgrad is a GEMM with K = pixels (dY^T x X_tap, one
 * warp per tap, partial sums per CTA reduced in a fixed order).
 *
 * This replaces the reference's learned operator model
 * (pararealml/operators/ml/supervised/supervised_ml_operator.py, sklearn /
 * keras regressors) with a convolutional network trained by these kernels.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "prml_internal.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int HC = 32;                      /* hidden channels */
constexpr int TR = 8, TC = 32;              /* tile: 8 rows x 32 columns of pixels */
constexpr int PR = TR + 2, PC = TC + 2;     /* with the 3x3 halo */
constexpr int PS = 40;                      /* bf16 per pixel in smem: 80 B, conflict-free ldmatrix */
constexpr int MID_SMEM = (PR * PC * PS + 9 * HC * PS) * (int)sizeof(bf16);
constexpr int WG_SMEM = (PR * PC * PS + TR * TC * PS) * (int)sizeof(bf16);

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 16 : 0)
               : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n cp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm_x4_t(unsigned (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0,
                                         unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

/* Stages the (TR+2) x (TC+2) pixel patch of 32 channels around the tile at
 * (y0, x0) of image b, zero outside the image. */
__device__ __forceinline__ void stage_patch(bf16* patch, const bf16* x, int b, int y0, int x0,
                                            int H, int W, int tid, int nthreads) {
  for (int i = tid; i < PR * PC * 4; i += nthreads) {
    const int pix = i >> 2, ch = i & 3;
    const int py = pix / PC, px = pix - py * PC;
    const int gy = y0 - 1 + py, gx = x0 - 1 + px;
    const bool ok = gy >= 0 && gy < H && gx >= 0 && gx < W;
    const bf16* src = ok ? x + ((((long long)b * H + gy) * W + gx) * HC + ch * 8) : x;
    cp_async16(patch + pix * PS + ch * 8, src, ok);
  }
}

/* 32 -> 32 3x3 convolution.  MODE 0: y = relu(conv(x, w) + bias).
 * MODE 1 (dgrad): y = conv(x, w) * (mask > 0), w given as [tap][ci][co]
 * with flipped taps by the caller.  w is [tap][n][k] (n = output channel). */
template <int MODE>
__global__ void __launch_bounds__(256) mid_conv(const bf16* __restrict__ x, const bf16* __restrict__ w,
                                                const float* __restrict__ bias,
                                                const bf16* __restrict__ mask, bf16* __restrict__ y,
                                                int B, int H, int W) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  bf16* patch = reinterpret_cast<bf16*>(smem_raw);
  bf16* wsm = patch + PR * PC * PS;
  const int tiles_c = (W + TC - 1) / TC, tiles_r = (H + TR - 1) / TR;
  const int per_img = tiles_c * tiles_r;
  const int b = blockIdx.x / per_img;
  const int r = blockIdx.x - b * per_img;
  const int y0 = (r / tiles_c) * TR, x0 = (r % tiles_c) * TC;
  const int tid = threadIdx.x;

  for (int i = tid; i < 9 * HC * 4; i += 256) {
    const int row = i >> 2, ch = i & 3;
    cp_async16(wsm + row * PS + ch * 8, w + row * HC + ch * 8, true);
  }
  stage_patch(patch, x, b, y0, x0, H, W, tid, 256);
  cp_async_wait_all();
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  const int gid = lane >> 2, tig = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[mt][nt][e] = 0.f;

#pragma unroll
  for (int tap = 0; tap < 9; ++tap) {
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
    for (int kk = 0; kk < 2; ++kk) {
      unsigned a[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int c = mt * 16 + (lane & 15);
        const int koff = kk * 16 + (lane >> 4) * 8;
        ldsm_x4(a[mt], patch + ((warp + 1 + dy) * PC + (c + 1 + dx)) * PS + koff);
      }
      unsigned bf[4][2];
#pragma unroll
      for (int np = 0; np < 2; ++np) {
        const int q = lane >> 3, i = lane & 7;
        const int co = (2 * np + (q >> 1)) * 8 + i;
        const int k = kk * 16 + (q & 1) * 8;
        unsigned t4[4];
        ldsm_x4(t4, wsm + (tap * HC + co) * PS + k);
        bf[2 * np][0] = t4[0];
        bf[2 * np][1] = t4[1];
        bf[2 * np + 1][0] = t4[2];
        bf[2 * np + 1][1] = t4[3];
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma16816(acc[mt][nt], a[mt], bf[nt][0], bf[nt][1]);
    }
  }

  const int gy = y0 + warp;
  if (gy >= H) return;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int gx = x0 + mt * 16 + gid + half * 8;
      if (gx >= W) continue;
      const long long p = ((long long)b * H + gy) * W + gx;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int co = nt * 8 + 2 * tig;
        float v0 = acc[mt][nt][half * 2], v1 = acc[mt][nt][half * 2 + 1];
        if (MODE == 0) {
          v0 = fmaxf(v0 + bias[co], 0.f);
          v1 = fmaxf(v1 + bias[co + 1], 0.f);
        } else {
          const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask + p * HC + co);
          v0 = __bfloat162float(mk.x) > 0.f ? v0 : 0.f;
          v1 = __bfloat162float(mk.y) > 0.f ? v1 : 0.f;
        }
        *reinterpret_cast<__nv_bfloat162*>(y + p * HC + co) = __floats2bfloat162_rn(v0, v1);
      }
    }
  }
}

/* dW[tap][co][ci] partial sums: sum over pixels of dy[p][co] * x[p + tap][ci].
 * One warp per tap (9 warps); each CTA walks tiles with a grid stride and
 * writes its partial [9][32][32] to partial + blockIdx.x * 9216. */
__global__ void __launch_bounds__(288) mid_wgrad(const bf16* __restrict__ x, const bf16* __restrict__ dy,
                                                 float* __restrict__ partial, int B, int H, int W) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  bf16* patch = reinterpret_cast<bf16*>(smem_raw);
  bf16* dsm = patch + PR * PC * PS;
  const int tiles_c = (W + TC - 1) / TC, tiles_r = (H + TR - 1) / TR;
  const int per_img = tiles_c * tiles_r;
  const long long total = (long long)per_img * B;
  const int tid = threadIdx.x;
  const int tap = tid >> 5, lane = tid & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int dyo = tap / 3 - 1, dxo = tap % 3 - 1;
  float acc[2][4][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[mt][nt][e] = 0.f;

  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    const int b = (int)(t / per_img);
    const int r = (int)(t - (long long)b * per_img);
    const int y0 = (r / tiles_c) * TR, x0 = (r % tiles_c) * TC;
    __syncthreads();
    stage_patch(patch, x, b, y0, x0, H, W, tid, 288);
    for (int i = tid; i < TR * TC * 4; i += 288) {
      const int pix = i >> 2, ch = i & 3;
      const int py = pix / TC, px = pix - py * TC;
      const int gy = y0 + py, gx = x0 + px;
      const bool ok = gy < H && gx < W;
      const bf16* src = ok ? dy + ((((long long)b * H + gy) * W + gx) * HC + ch * 8) : dy;
      cp_async16(dsm + pix * PS + ch * 8, src, ok);
    }
    cp_async_wait_all();
    __syncthreads();
#pragma unroll 4
    for (int ks = 0; ks < TR * TC / 16; ++ks) {
      const int row = ks >> 1, h = ks & 1;
      const int q = lane >> 3, i = lane & 7;
      unsigned a[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int px = h * 16 + (q >> 1) * 8 + i;
        const int co = mt * 16 + (q & 1) * 8;
        ldsm_x4_t(a[mt], dsm + (row * TC + px) * PS + co);
      }
      unsigned bf[4][2];
#pragma unroll
      for (int np = 0; np < 2; ++np) {
        const int px = h * 16 + (q & 1) * 8 + i;
        const int ci = (2 * np + (q >> 1)) * 8;
        unsigned t4[4];
        ldsm_x4_t(t4, patch + ((row + 1 + dyo) * PC + (px + 1 + dxo)) * PS + ci);
        bf[2 * np][0] = t4[0];
        bf[2 * np][1] = t4[1];
        bf[2 * np + 1][0] = t4[2];
        bf[2 * np + 1][1] = t4[3];
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma16816(acc[mt][nt], a[mt], bf[nt][0], bf[nt][1]);
    }
  }
  float* out = partial + (long long)blockIdx.x * 9 * HC * HC + tap * HC * HC;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int co = mt * 16 + gid, ci = nt * 8 + 2 * tig;
      out[co * HC + ci] = acc[mt][nt][0];
      out[co * HC + ci + 1] = acc[mt][nt][1];
      out[(co + 8) * HC + ci] = acc[mt][nt][2];
      out[(co + 8) * HC + ci + 1] = acc[mt][nt][3];
    }
}

/* out[i] = scale * sum_k partial[k * n + i]: a (32, 8) block per 32 outputs,
 * row ty sums the parts k = ty (mod 8), then the 8 row sums are added in
 * order (deterministic for a given part count). */
__global__ void __launch_bounds__(256) reduce_parts(const float* __restrict__ partial, int parts, int n,
                                                    float* __restrict__ out, float scale) {
  __shared__ float red[8][32];
  const int i = blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (i < n)
    for (int k = threadIdx.y; k < parts; k += 8) s += partial[(long long)k * n + i];
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && i < n) {
    float t = 0.f;
#pragma unroll
    for (int r = 0; r < 8; ++r) t += red[r][threadIdx.x];
    out[i] = t * scale;
  }
}

/* [9][co][ci] -> [9][ci][co] (the wgrad GEMM's output is co-major) */
__global__ void wgrad_transpose(const float* __restrict__ in, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 9 * HC * HC) return;
  const int t = i / (HC * HC), r = i % (HC * HC);
  const int co = r / HC, ci = r % HC;
  out[t * HC * HC + ci * HC + co] = in[i];
}

template <typename S>
__device__ __forceinline__ float state_at(const S* u, int b, int c, int y, int x, int H, int W,
                                          int pitch) {
  if (y < 0 || y >= H || x < 0 || x >= W) return 0.f;
  return (float)u[(((long long)b * 2 + c) * H + y) * pitch + x];
}

/* Packs 8 floats (after ReLU when RELU) into 8 bf16 (round to nearest). */
template <bool RELU>
__device__ __forceinline__ uint4 pack8(const float* v) {
  uint4 r;
  unsigned* w = reinterpret_cast<unsigned*>(&r);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float a = RELU ? fmaxf(v[2 * k], 0.f) : v[2 * k];
    const float b = RELU ? fmaxf(v[2 * k + 1], 0.f) : v[2 * k + 1];
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    w[k] = *reinterpret_cast<const unsigned*>(&h);
  }
  return r;
}

/* The 2 -> 32 layers (in_fwd) and the 32 -> 2 layer's data gradient
 * (out_dgrad) take 8 x 64 pixel tiles: the 10 x 66 halo tile of both
 * 2-channel planes is staged as float in shared memory (zero outside the
 * image), warp w computes tile row w and lane l its pixels l and l + 32, all
 * 32 channels, reading the weights of 4 channels as one 16-byte shared load
 * used for both pixels.  Each output is the same sum, in the same order, as
 * one thread per pixel reading every operand separately. */
constexpr int TL_TR = 8, TL_TW = 64;

/* x1 = relu(conv3x3(s_in * u; w0 [9][2][32]) + b0) */
template <typename S>
__global__ void __launch_bounds__(256, 2) in_fwd(const S* __restrict__ u, int pitch, const float* __restrict__ w0,
                                                 const float* __restrict__ b0, const float* __restrict__ s_in,
                                                 bf16* __restrict__ x1, int B, int H, int W) {
  __shared__ __align__(16) float ws[9 * 2 * HC + HC];
  __shared__ float us[2][TL_TR + 2][TL_TW + 2];
  for (int i = threadIdx.x; i < 9 * 2 * HC; i += blockDim.x) ws[i] = w0[i] * s_in[(i / HC) & 1];
  for (int i = threadIdx.x; i < HC; i += blockDim.x) ws[9 * 2 * HC + i] = b0[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ntx = (W + TL_TW - 1) / TL_TW, nty = (H + TL_TR - 1) / TL_TR;
  const long long ntiles = (long long)B * nty * ntx;
  for (long long it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const int b = (int)(it / ((long long)nty * ntx));
    const int rem = (int)(it - (long long)b * nty * ntx);
    const int y0 = (rem / ntx) * TL_TR, x0 = (rem % ntx) * TL_TW;
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * (TL_TR + 2) * (TL_TW + 2); e += blockDim.x) {
      const int c = e / ((TL_TR + 2) * (TL_TW + 2));
      const int r = (e / (TL_TW + 2)) % (TL_TR + 2), col = e % (TL_TW + 2);
      us[c][r][col] = state_at(u, b, c, y0 + r - 1, x0 + col - 1, H, W, pitch);
    }
    __syncthreads();
    const int y = y0 + warp;
    if (y >= H || x0 + lane >= W) continue;
    float acc0[HC], acc1[HC];
#pragma unroll
    for (int co = 0; co < HC; ++co) acc0[co] = acc1[co] = ws[9 * 2 * HC + co];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const float a0 = us[0][warp + t / 3][lane + t % 3], a1 = us[1][warp + t / 3][lane + t % 3];
      const float c0 = us[0][warp + t / 3][lane + 32 + t % 3], c1 = us[1][warp + t / 3][lane + 32 + t % 3];
      const float4* wa = reinterpret_cast<const float4*>(ws + (t * 2 + 0) * HC);
      const float4* wb = reinterpret_cast<const float4*>(ws + (t * 2 + 1) * HC);
#pragma unroll
      for (int k = 0; k < HC / 4; ++k) {
        const float4 p = wa[k], q = wb[k];
        acc0[4 * k + 0] += a0 * p.x + a1 * q.x;
        acc0[4 * k + 1] += a0 * p.y + a1 * q.y;
        acc0[4 * k + 2] += a0 * p.z + a1 * q.z;
        acc0[4 * k + 3] += a0 * p.w + a1 * q.w;
        acc1[4 * k + 0] += c0 * p.x + c1 * q.x;
        acc1[4 * k + 1] += c0 * p.y + c1 * q.y;
        acc1[4 * k + 2] += c0 * p.z + c1 * q.z;
        acc1[4 * k + 3] += c0 * p.w + c1 * q.w;
      }
    }
    const long long p0 = ((long long)b * H + y) * W + x0 + lane;
    uint4* d0 = reinterpret_cast<uint4*>(x1 + p0 * HC);
#pragma unroll
    for (int q = 0; q < HC / 8; ++q) d0[q] = pack8<true>(acc0 + 8 * q);
    if (x0 + lane + 32 < W) {
      uint4* d1 = reinterpret_cast<uint4*>(x1 + (p0 + 32) * HC);
#pragma unroll
      for (int q = 0; q < HC / 8; ++q) d1[q] = pack8<true>(acc1 + 8 * q);
    }
  }
}

/* y = u + s_out * (conv3x3(x5; w5 [9][32][2]) + b5).
 * A CTA stages the (TR+2) x (TW+2) pixel tile of x5 around its TR x TW
 * output tile in shared memory with 16-byte loads, one pixel every 80 bytes
 * (32 bf16 + 16 pad): 8 consecutive lanes reading 16 bytes each then hit
 * distinct banks.  Warp w computes tile rows 2w and 2w + 1 (lanes 0-15 and
 * 16-31), lane l the pixels l mod 16 and l mod 16 + 16 of its row; the
 * weights of two input channels for both outputs are one 16-byte shared
 * load used for both pixels.  Each output is the same sum, in the same
 * order, as one thread per pixel reading every weight separately. */
constexpr int OUTF_TW = 32, OUTF_TR = 8, OUTF_PS = HC + 8, OUTF_THREADS = 128;

template <typename S>
__global__ void __launch_bounds__(OUTF_THREADS) out_fwd(const bf16* __restrict__ x5, const float* __restrict__ w5,
                                                        const float* __restrict__ b5, const float* __restrict__ s_out,
                                                        const S* __restrict__ u, S* __restrict__ yout, int pitch,
                                                        int B, int H, int W) {
  __shared__ __align__(16) float ws[9 * HC * 2];
  __shared__ __align__(16) bf16 xs[(OUTF_TR + 2) * (OUTF_TW + 2) * OUTF_PS];
  for (int i = threadIdx.x; i < 9 * HC * 2; i += blockDim.x) ws[i] = w5[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int lx = lane & 15, ly = 2 * warp + (lane >> 4);
  const int ntx = (W + OUTF_TW - 1) / OUTF_TW, nty = (H + OUTF_TR - 1) / OUTF_TR;
  const long long ntiles = (long long)B * nty * ntx;
  const float bias0 = b5[0], bias1 = b5[1], so0 = s_out[0], so1 = s_out[1];
  const float4* w4 = reinterpret_cast<const float4*>(ws);
  for (long long it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const int b = (int)(it / ((long long)nty * ntx));
    const int rem = (int)(it - (long long)b * nty * ntx);
    const int y0 = (rem / ntx) * OUTF_TR, x0 = (rem % ntx) * OUTF_TW;
    __syncthreads();
    for (int e = threadIdx.x; e < (OUTF_TR + 2) * (OUTF_TW + 2) * 4; e += blockDim.x) {
      const int pix = e >> 2, q = e & 3;
      const int yy = y0 + pix / (OUTF_TW + 2) - 1, xx = x0 + pix % (OUTF_TW + 2) - 1;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (yy >= 0 && yy < H && xx >= 0 && xx < W)
        v = *reinterpret_cast<const uint4*>(x5 + (((long long)b * H + yy) * W + xx) * HC + q * 8);
      *reinterpret_cast<uint4*>(xs + pix * OUTF_PS + q * 8) = v;
    }
    __syncthreads();
    const int y = y0 + ly, x = x0 + lx;
    if (y >= H || x >= W) continue;
    float z0 = bias0, z1 = bias1, z2 = bias0, z3 = bias1; /* pixel x: z0, z1; pixel x + 16: z2, z3 */
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const bf16* sa = xs + ((ly + t / 3) * (OUTF_TW + 2) + lx + t % 3) * OUTF_PS;
      const bf16* sb = sa + 16 * OUTF_PS;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint4 ra = *reinterpret_cast<const uint4*>(sa + q * 8);
        const uint4 rb = *reinterpret_cast<const uint4*>(sb + q * 8);
        const __nv_bfloat162* ha = reinterpret_cast<const __nv_bfloat162*>(&ra);
        const __nv_bfloat162* hb = reinterpret_cast<const __nv_bfloat162*>(&rb);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float2 va = __bfloat1622float2(ha[j]), vb = __bfloat1622float2(hb[j]);
          /* (w[ci][0], w[ci][1], w[ci+1][0], w[ci+1][1]), ci = q * 8 + 2 j */
          const float4 w = w4[(t * HC + q * 8 + 2 * j) / 2];
          z0 += va.x * w.x + va.y * w.z;
          z1 += va.x * w.y + va.y * w.w;
          z2 += vb.x * w.x + vb.y * w.z;
          z3 += vb.x * w.y + vb.y * w.w;
        }
      }
    }
    const long long o0 = (((long long)b * 2 + 0) * H + y) * pitch + x;
    const long long o1 = (((long long)b * 2 + 1) * H + y) * pitch + x;
    yout[o0] = (S)((float)u[o0] + so0 * z0);
    yout[o1] = (S)((float)u[o1] + so1 * z1);
    if (x + 16 < W) {
      yout[o0 + 16] = (S)((float)u[o0 + 16] + so0 * z2);
      yout[o1 + 16] = (S)((float)u[o1 + 16] + so1 * z3);
    }
  }
}

/* dx5 = (conv^T(g; w5)) * (x5 > 0), g = dy * s_out (dy dense fp32 [B][2][H][W]);
 * the 8 x 64 tiles of in_fwd, the staged planes holding dy. */
__global__ void __launch_bounds__(256, 2) out_dgrad(const float* __restrict__ dy, const bf16* __restrict__ x5,
                                                    const float* __restrict__ w5, const float* __restrict__ s_out,
                                                    bf16* __restrict__ dx5, int B, int H, int W) {
  __shared__ __align__(16) float ws[9 * HC * 2];
  __shared__ float gs[2][TL_TR + 2][TL_TW + 2];
  for (int i = threadIdx.x; i < 9 * HC * 2; i += blockDim.x) ws[i] = w5[i] * s_out[i & 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ntx = (W + TL_TW - 1) / TL_TW, nty = (H + TL_TR - 1) / TL_TR;
  const long long ntiles = (long long)B * nty * ntx;
  const float4* w4 = reinterpret_cast<const float4*>(ws);
  for (long long it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const int b = (int)(it / ((long long)nty * ntx));
    const int rem = (int)(it - (long long)b * nty * ntx);
    const int y0 = (rem / ntx) * TL_TR, x0 = (rem % ntx) * TL_TW;
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * (TL_TR + 2) * (TL_TW + 2); e += blockDim.x) {
      const int c = e / ((TL_TR + 2) * (TL_TW + 2));
      const int r = (e / (TL_TW + 2)) % (TL_TR + 2), col = e % (TL_TW + 2);
      const int yy = y0 + r - 1, xx = x0 + col - 1;
      gs[c][r][col] = (yy >= 0 && yy < H && xx >= 0 && xx < W) ? dy[(((long long)b * 2 + c) * H + yy) * W + xx] : 0.f;
    }
    __syncthreads();
    const int y = y0 + warp;
    if (y >= H || x0 + lane >= W) continue;
    float acc0[HC], acc1[HC];
#pragma unroll
    for (int ci = 0; ci < HC; ++ci) acc0[ci] = acc1[ci] = 0.f;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      /* tap t reads g at (y - (t / 3 - 1), x - (t % 3 - 1)); outside the
       * image the staged zeros add nothing (the sums start at +0) */
      const int r = warp + 2 - t / 3, c = lane + 2 - t % 3;
      const float a0 = gs[0][r][c], a1 = gs[1][r][c];
      const float c0 = gs[0][r][c + 32], c1 = gs[1][r][c + 32];
#pragma unroll
      for (int ci = 0; ci < HC; ci += 2) {
        /* (w[ci][0], w[ci][1], w[ci+1][0], w[ci+1][1]) */
        const float4 w = w4[(t * HC + ci) / 2];
        acc0[ci] += a0 * w.x + a1 * w.y;
        acc0[ci + 1] += a0 * w.z + a1 * w.w;
        acc1[ci] += c0 * w.x + c1 * w.y;
        acc1[ci + 1] += c0 * w.z + c1 * w.w;
      }
    }
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int x = x0 + lane + 32 * half;
      if (x >= W) break;
      const long long p = ((long long)b * H + y) * W + x;
      const float* acc = half ? acc1 : acc0;
      const uint4* m4 = reinterpret_cast<const uint4*>(x5 + p * HC);
      uint4* d4 = reinterpret_cast<uint4*>(dx5 + p * HC);
#pragma unroll
      for (int q = 0; q < HC / 8; ++q) {
        const uint4 mr = m4[q];
        const __nv_bfloat162* mh = reinterpret_cast<const __nv_bfloat162*>(&mr);
        float v[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float2 m = __bfloat1622float2(mh[k]);
          v[2 * k] = m.x > 0.f ? acc[8 * q + 2 * k] : 0.f;
          v[2 * k + 1] = m.y > 0.f ? acc[8 * q + 2 * k + 1] : 0.f;
        }
        d4[q] = pack8<false>(v);
      }
    }
  }
}

/* Thin-layer weight gradients, both a sum over pixels p of A[p][a] * S[p + tap][b]:
 *   OUT = 0 (input layer):  dW0[t][ci][co] = sum g1[p][co] * s_in[ci] u[p+t][ci],
 *                           A = g1 (bf16 NHWC gradient of x1, 32 ch), S = s_in * u (2 ch);
 *   OUT = 1 (output layer): dW5[t][ci][co] = sum s_out[co] dy[p][co] * x5[p+t][ci],
 *                           A = s_out * dy (2 ch), S = x5 (bf16 NHWC, 32 ch).
 * A CTA stages a TR x TW pixel tile of A and the (TR+2) x (TW+2) tile of S
 * around it in shared memory (zero outside the image; the 32-channel operand
 * stays bf16 and moves in 16-byte loads).  Each of its 256 threads owns one
 * (co, ci) pair and the tile rows r = 4k + row: it slides a 3x3 window of S
 * along each row and accumulates all 9 taps.  Lanes run over the 32-channel
 * operand, so its reads are conflict-free and the 2-channel reads broadcast.
 * Bias gradients are the plain sums of A.  The 4 row-class partials are summed
 * in shared memory and each CTA writes one partial row (weights, then biases). */
constexpr int THIN_TW = 32, THIN_TR = 8;

template <int OUT>
__device__ __forceinline__ float thin_a(const float* sa2, const bf16* sa32, int r, int x, int c) {
  return OUT ? sa2[(r * THIN_TW + x) * 2 + c] : __bfloat162float(sa32[(r * THIN_TW + x) * HC + c]);
}

template <int OUT>
__device__ __forceinline__ float thin_s(const float* ss2, const bf16* ss32, int r, int x, int c) {
  return OUT ? __bfloat162float(ss32[(r * (THIN_TW + 2) + x) * HC + c]) : ss2[(r * (THIN_TW + 2) + x) * 2 + c];
}

/* 16-byte chunks of a bf16 NHWC tile: rows y0.., cols x0.. (zero outside). */
__device__ __forceinline__ void thin_stage32(const bf16* __restrict__ g, bf16* dst, int b, int y0, int x0,
                                             int rows, int cols, int H, int W) {
  for (int e = threadIdx.x; e < rows * cols * 4; e += blockDim.x) {
    const int pix = e >> 2, q = e & 3;
    const int yy = y0 + pix / cols, xx = x0 + pix % cols;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (yy >= 0 && yy < H && xx >= 0 && xx < W)
      v = *reinterpret_cast<const uint4*>(g + (((long long)b * H + yy) * W + xx) * HC + q * 8);
    *reinterpret_cast<uint4*>(dst + pix * HC + q * 8) = v;
  }
}

template <int OUT, typename S>
__global__ void __launch_bounds__(256) thin_wgrad(const bf16* __restrict__ g1, const S* __restrict__ u,
                                                  int pitch, const float* __restrict__ s_in,
                                                  const float* __restrict__ dy, const bf16* __restrict__ x5,
                                                  const float* __restrict__ s_out, float* __restrict__ partial,
                                                  int B, int H, int W) {
  constexpr int CA = OUT ? 2 : HC;
  constexpr int NW = 9 * 2 * HC;
  constexpr int NK = NW + CA;
  constexpr int A_ELEMS = THIN_TR * THIN_TW * CA;
  constexpr int S_ELEMS = (THIN_TR + 2) * (THIN_TW + 2) * (OUT ? HC : 2);
  __shared__ __align__(16) bf16 s32[OUT ? S_ELEMS : A_ELEMS];
  __shared__ float s2[OUT ? A_ELEMS : S_ELEMS];
  __shared__ float red[4][NK];
  const float* sa2 = s2;
  const float* ss2 = s2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int two = warp & 1, row = warp >> 1;
  const int ia = OUT ? two : lane;  /* channel of A (co) */
  const int is = OUT ? lane : two;  /* channel of S (ci) */
  const int ntx = (W + THIN_TW - 1) / THIN_TW, nty = (H + THIN_TR - 1) / THIN_TR;
  const long long ntiles = (long long)B * nty * ntx;
  float acc[9];
#pragma unroll
  for (int t = 0; t < 9; ++t) acc[t] = 0.f;
  float bsum = 0.f;
  for (long long it = blockIdx.x; it < ntiles; it += gridDim.x) {
    const int b = (int)(it / ((long long)nty * ntx));
    const int rem = (int)(it - (long long)b * nty * ntx);
    const int y0 = (rem / ntx) * THIN_TR, x0 = (rem % ntx) * THIN_TW;
    __syncthreads();
    if (OUT == 0) {
      thin_stage32(g1, s32, b, y0, x0, THIN_TR, THIN_TW, H, W);
      for (int e = threadIdx.x; e < S_ELEMS; e += 256) {
        const int x = e % (THIN_TW + 2), r = (e / (THIN_TW + 2)) % (THIN_TR + 2), c = e / ((THIN_TW + 2) * (THIN_TR + 2));
        s2[(r * (THIN_TW + 2) + x) * 2 + c] = s_in[c] * state_at(u, b, c, y0 + r - 1, x0 + x - 1, H, W, pitch);
      }
    } else {
      for (int e = threadIdx.x; e < A_ELEMS; e += 256) {
        const int x = e % THIN_TW, r = (e / THIN_TW) % THIN_TR, c = e / (THIN_TW * THIN_TR);
        const int yy = y0 + r, xx = x0 + x;
        s2[(r * THIN_TW + x) * 2 + c] = (yy < H && xx < W) ? s_out[c] * dy[(((long long)b * 2 + c) * H + yy) * W + xx] : 0.f;
      }
      thin_stage32(x5, s32, b, y0 - 1, x0 - 1, THIN_TR + 2, THIN_TW + 2, H, W);
    }
    __syncthreads();
#pragma unroll
    for (int rk = 0; rk < THIN_TR / 4; ++rk) {
      const int r = rk * 4 + row;
      float win[3][3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        win[d][0] = 0.f;
        win[d][1] = thin_s<OUT>(ss2, s32, r + d, 0, is);
        win[d][2] = thin_s<OUT>(ss2, s32, r + d, 1, is);
      }
#pragma unroll 4
      for (int x = 0; x < THIN_TW; ++x) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          win[d][0] = win[d][1];
          win[d][1] = win[d][2];
          win[d][2] = thin_s<OUT>(ss2, s32, r + d, x + 2, is);
        }
        const float av = thin_a<OUT>(sa2, s32, r, x, ia);
        bsum += av;
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int e = 0; e < 3; ++e) acc[d * 3 + e] = fmaf(av, win[d][e], acc[d * 3 + e]);
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < 9; ++t) red[row][t * 2 * HC + (OUT ? is * 2 + ia : is * HC + ia)] = acc[t];
  if (is == 0) red[row][NW + ia] = bsum;
  __syncthreads();
  for (int k = threadIdx.x; k < NK; k += 256) {
    float s = 0.f;
#pragma unroll
    for (int r = 0; r < 4; ++r) s += red[r][k];
    partial[(long long)blockIdx.x * NK + k] = s;
  }
}

/* Bias gradient of a hidden layer: sum over pixels of g[p][co]. */
__global__ void __launch_bounds__(256) channel_sum(const bf16* __restrict__ g, long long npix,
                                                   float* __restrict__ partial) {
  __shared__ float red[8][HC];
  const int c = threadIdx.x & 31, lane_row = threadIdx.x >> 5;
  const long long per = (npix + gridDim.x - 1) / gridDim.x;
  const long long lo = blockIdx.x * per, hi = lo + per < npix ? lo + per : npix;
  float s = 0.f;
  for (long long p = lo + lane_row; p < hi; p += 8) s += __bfloat162float(g[p * HC + c]);
  red[lane_row][c] = s;
  __syncthreads();
  if (threadIdx.x < HC) {
    float t = 0.f;
    for (int r = 0; r < 8; ++r) t += red[r][threadIdx.x];
    partial[(long long)blockIdx.x * HC + threadIdx.x] = t;
  }
}

/* dy = 2 (y - target) / n (dense fp32 [B][2][H][W]); partial[block] = sum of squares. */
template <typename S>
__global__ void __launch_bounds__(256) mse_grad(const S* __restrict__ y, const S* __restrict__ target,
                                                int pitch, int B, int H, int W, float* __restrict__ dy,
                                                double* __restrict__ partial) {
  const long long n = (long long)B * 2 * H * W;
  const float scale = (float)(2.0 / (double)n);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double s = 0.0;
  for (long long row = blockIdx.x * 8LL + warp; row < (long long)B * 2 * H; row += gridDim.x * 8LL) {
    const S* yr = y + row * pitch;
    const S* tr = target + row * pitch;
    float* dr = dy + row * W;
    for (int x = lane; x < W; x += 32) {
      const S d = yr[x] - tr[x];
      dr[x] = (float)d * scale;
      s += (double)d * (double)d;
    }
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

/* Adam on fp32 master parameters. */
__global__ void adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                     float* __restrict__ v, long long n, float lr, float b1, float b2, float eps,
                     float bc1, float bc2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

/* w [9][ci][co] fp32 -> forward bf16 [9][co][ci] and dgrad bf16 [9][ci][co]
 * with flipped taps (tap' = 8 - tap). */
__global__ void pack_mid(const float* __restrict__ w, bf16* __restrict__ wf, bf16* __restrict__ wd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 9 * HC * HC) return;
  const int t = i / (HC * HC), r = i % (HC * HC);
  const int ci = r / HC, co = r % HC;
  const bf16 v = __float2bfloat16_rn(w[i]);
  wf[(t * HC + co) * HC + ci] = v;
  wd[((8 - t) * HC + ci) * HC + co] = v;
}

int grid_pix(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

/* CTAs of a tile-walking kernel: one per tile, at most 16 per SM. */
int grid_tiles(int B, int H, int W, int tr, int tw) {
  long long g = (long long)B * ((H + tr - 1) / tr) * ((W + tw - 1) / tw);
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

int last(const char* what) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PRML_OK : prml_set_error(PRML_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool g_attrs_set = false;

int set_attrs() {
  if (g_attrs_set) return PRML_OK;
  cudaError_t e = cudaFuncSetAttribute(mid_conv<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, MID_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(mid_conv<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, MID_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(mid_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, WG_SMEM);
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("cnn attributes: ") + cudaGetErrorString(e));
  g_attrs_set = true;
  return PRML_OK;
}

bool check_dims(int B, int H, int W) { return B >= 1 && H >= 1 && W >= 1; }

}  // namespace

extern "C" {

int prml_cnn_in_fwd(const void* u, int elem_bytes, int pitch, const float* w0, const float* b0,
                    const float* s_in, void* x1, int B, int H, int W, void* stream) {
  if (!u || !w0 || !b0 || !s_in || !x1 || !check_dims(B, H, W) || pitch < W)
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_in_fwd: bad argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int g = grid_tiles(B, H, W, TL_TR, TL_TW);
  if (elem_bytes == 4)
    in_fwd<float><<<g, 256, 0, s>>>(static_cast<const float*>(u), pitch, w0, b0, s_in, static_cast<bf16*>(x1), B, H, W);
  else if (elem_bytes == 8)
    in_fwd<double><<<g, 256, 0, s>>>(static_cast<const double*>(u), pitch, w0, b0, s_in, static_cast<bf16*>(x1), B, H, W);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_in_fwd: elem_bytes must be 4 or 8");
  return last("prml_cnn_in_fwd");
}

int prml_cnn_mid_fwd(const void* x, const void* wf, const float* bias, void* y, int B, int H, int W,
                     void* stream) {
  if (!x || !wf || !bias || !y || !check_dims(B, H, W))
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_mid_fwd: bad argument");
  if (prml_cnn_tc_enabled()) return prml_cnn_mid_conv_tc(0, x, wf, bias, nullptr, y, B, H, W, stream);
  int rc = set_attrs();
  if (rc) return rc;
  const long long tiles = (long long)B * ((H + TR - 1) / TR) * ((W + TC - 1) / TC);
  if (tiles > 0x7fffffffLL) return prml_set_error(PRML_ERR_ARG, "prml_cnn_mid_fwd: too many tiles");
  mid_conv<0><<<(unsigned)tiles, 256, MID_SMEM, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(x), static_cast<const bf16*>(wf), bias, nullptr, static_cast<bf16*>(y), B, H, W);
  return last("prml_cnn_mid_fwd");
}

int prml_cnn_mid_dgrad(const void* g, const void* wd, const void* mask, void* gx, int B, int H, int W,
                       void* stream) {
  if (!g || !wd || !mask || !gx || !check_dims(B, H, W))
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_mid_dgrad: bad argument");
  if (prml_cnn_tc_enabled()) return prml_cnn_mid_conv_tc(1, g, wd, nullptr, mask, gx, B, H, W, stream);
  int rc = set_attrs();
  if (rc) return rc;
  const long long tiles = (long long)B * ((H + TR - 1) / TR) * ((W + TC - 1) / TC);
  mid_conv<1><<<(unsigned)tiles, 256, MID_SMEM, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(g), static_cast<const bf16*>(wd), nullptr, static_cast<const bf16*>(mask),
      static_cast<bf16*>(gx), B, H, W);
  return last("prml_cnn_mid_dgrad");
}

long long prml_cnn_wgrad_scratch_elems(int parts) { return (long long)parts * 9 * HC * HC + 9 * HC * HC; }

int prml_cnn_mid_wgrad(const void* x, const void* g, float* dw, float* db, int parts, float* scratch,
                       int B, int H, int W, void* stream) {
  if (!x || !g || !dw || !db || !scratch || parts < 1 || !check_dims(B, H, W))
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_mid_wgrad: bad argument");
  int rc = set_attrs();
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int n = 9 * HC * HC;
  float* co_major = scratch + (long long)parts * n;
  int used = parts;
  if (prml_cnn_tc_enabled()) {
    rc = prml_cnn_mid_wgrad_tc(x, g, scratch, parts, &used, B, H, W, stream);
    if (rc) return rc;
  } else {
    mid_wgrad<<<parts, 288, WG_SMEM, s>>>(static_cast<const bf16*>(x), static_cast<const bf16*>(g), scratch, B, H, W);
  }
  reduce_parts<<<(n + 31) / 32, dim3(32, 8), 0, s>>>(scratch, used, n, co_major, 1.f);
  wgrad_transpose<<<(n + 255) / 256, 256, 0, s>>>(co_major, dw);
  channel_sum<<<parts, 256, 0, s>>>(static_cast<const bf16*>(g), (long long)B * H * W, scratch);
  reduce_parts<<<1, dim3(32, 8), 0, s>>>(scratch, parts, HC, db, 1.f);
  return last("prml_cnn_mid_wgrad");
}

int prml_cnn_out_fwd(const void* x5, const float* w5, const float* b5, const float* s_out,
                     const void* u, void* y, int elem_bytes, int pitch, int B, int H, int W,
                     void* stream) {
  if (!x5 || !w5 || !b5 || !s_out || !u || !y || !check_dims(B, H, W) || pitch < W)
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_out_fwd: bad argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int g = grid_tiles(B, H, W, OUTF_TR, OUTF_TW);
  if (elem_bytes == 4)
    out_fwd<float><<<g, OUTF_THREADS, 0, s>>>(static_cast<const bf16*>(x5), w5, b5, s_out, static_cast<const float*>(u),
                                     static_cast<float*>(y), pitch, B, H, W);
  else if (elem_bytes == 8)
    out_fwd<double><<<g, OUTF_THREADS, 0, s>>>(static_cast<const bf16*>(x5), w5, b5, s_out, static_cast<const double*>(u),
                                      static_cast<double*>(y), pitch, B, H, W);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_out_fwd: elem_bytes must be 4 or 8");
  return last("prml_cnn_out_fwd");
}

int prml_cnn_out_bwd(const float* dy, const void* x5, const float* w5, const float* s_out, void* dx5,
                     float* dw5, float* db5, int parts, float* scratch, int B, int H, int W,
                     void* stream) {
  if (!dy || !x5 || !w5 || !s_out || !dx5 || !dw5 || !db5 || !scratch || parts < 1 || !check_dims(B, H, W))
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_out_bwd: bad argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  out_dgrad<<<grid_tiles(B, H, W, TL_TR, TL_TW), 256, 0, s>>>(dy, static_cast<const bf16*>(x5), w5, s_out,
                                                               static_cast<bf16*>(dx5), B, H, W);
  const int nk = 9 * 2 * HC + 2;
  thin_wgrad<1, float><<<parts, 256, 0, s>>>(nullptr, nullptr, 0, nullptr, dy, static_cast<const bf16*>(x5),
                                             s_out, scratch, B, H, W);
  reduce_parts<<<(nk + 31) / 32, dim3(32, 8), 0, s>>>(scratch, parts, nk, scratch + (long long)parts * nk, 1.f);
  cudaMemcpyAsync(dw5, scratch + (long long)parts * nk, 9 * 2 * HC * sizeof(float), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(db5, scratch + (long long)parts * nk + 9 * 2 * HC, 2 * sizeof(float), cudaMemcpyDeviceToDevice, s);
  return last("prml_cnn_out_bwd");
}

int prml_cnn_in_wgrad(const void* g1, const void* u, int elem_bytes, int pitch, const float* s_in,
                      float* dw0, float* db0, int parts, float* scratch, int B, int H, int W,
                      void* stream) {
  if (!g1 || !u || !s_in || !dw0 || !db0 || !scratch || parts < 1 || !check_dims(B, H, W) || pitch < W)
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_in_wgrad: bad argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nk = 9 * 2 * HC + HC;
  if (elem_bytes == 4)
    thin_wgrad<0, float><<<parts, 256, 0, s>>>(static_cast<const bf16*>(g1), static_cast<const float*>(u), pitch,
                                               s_in, nullptr, nullptr, nullptr, scratch, B, H, W);
  else if (elem_bytes == 8)
    thin_wgrad<0, double><<<parts, 256, 0, s>>>(static_cast<const bf16*>(g1), static_cast<const double*>(u), pitch,
                                                s_in, nullptr, nullptr, nullptr, scratch, B, H, W);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_in_wgrad: elem_bytes must be 4 or 8");
  reduce_parts<<<(nk + 31) / 32, dim3(32, 8), 0, s>>>(scratch, parts, nk, scratch + (long long)parts * nk, 1.f);
  cudaMemcpyAsync(dw0, scratch + (long long)parts * nk, 9 * 2 * HC * sizeof(float), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(db0, scratch + (long long)parts * nk + 9 * 2 * HC, HC * sizeof(float), cudaMemcpyDeviceToDevice, s);
  return last("prml_cnn_in_wgrad");
}

long long prml_cnn_thin_scratch_elems(int parts) { return (long long)(parts + 1) * (9 * 2 * HC + HC); }

int prml_cnn_mse(const void* y, const void* target, int elem_bytes, int pitch, int B, int H, int W,
                 float* dy, double* partial, int parts, void* stream) {
  if (!y || !target || !dy || !partial || parts < 1 || !check_dims(B, H, W) || pitch < W)
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_mse: bad argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (elem_bytes == 4)
    mse_grad<float><<<parts, 256, 0, s>>>(static_cast<const float*>(y), static_cast<const float*>(target), pitch, B,
                                          H, W, dy, partial);
  else if (elem_bytes == 8)
    mse_grad<double><<<parts, 256, 0, s>>>(static_cast<const double*>(y), static_cast<const double*>(target), pitch,
                                           B, H, W, dy, partial);
  else
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_mse: elem_bytes must be 4 or 8");
  return last("prml_cnn_mse");
}

int prml_cnn_adam(float* params, const float* grads, float* m, float* v, long long n, float lr,
                  float beta1, float beta2, float eps, int step, void* stream) {
  if (!params || !grads || !m || !v || n < 1 || step < 1)
    return prml_set_error(PRML_ERR_ARG, "prml_cnn_adam: bad argument");
  const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
  adam<<<grid_pix(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(params, grads, m, v, n, lr, beta1, beta2,
                                                                         eps, bc1, bc2);
  return last("prml_cnn_adam");
}

int prml_cnn_pack_mid(const float* w, void* wf, void* wd, void* stream) {
  if (!w || !wf || !wd) return prml_set_error(PRML_ERR_ARG, "prml_cnn_pack_mid: bad argument");
  pack_mid<<<(9 * HC * HC + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      w, static_cast<bf16*>(wf), static_cast<bf16*>(wd));
  return last("prml_cnn_pack_mid");
}

}  // extern "C"
