/*
 * 32 -> 32 channel 3x3 convolutions of the residual CNN on the 5th-generation
 * tensor cores (tcgen05, accumulators in tensor memory).
 *
 * Implicit GEMM per tile: M = 128 pixels (one row segment of one image),
 * N = 32 output channels, K = 9 taps x 32 input channels, issued as
 * 18 tcgen05.mma.kind::f16 (bf16 x bf16 -> f32, M128 N32 K16).
 *
 * Work item: a band of up to 16 output rows of one 128-pixel column segment.
 * A CTA walks down the band; the input rows stream through a ring of 8
 * staged rows, so each output row costs one new input row: ONE TMA box load
 * of 130 whole pixels (64 bytes each, zero filled outside the image) with
 * the 64-byte swizzle.  That is the SWIZZLE_64B K-major canonical layout
 * (rows of 64 bytes = all 32 input channels, 8-row groups 512 bytes apart),
 * so the A matrix of tap (dy, dx) and K half kk starts at pixel dx, byte
 * 32 kk of the row for dy.  B operand: the packed weights [tap][n][k],
 * staged once per CTA as [tap][chunk][n][8] (no swizzle).
 *
 * Roles per CTA (320 threads): warp 8 issues the row loads, warp 9 issues
 * the MMAs into one of four 32-column TMEM accumulators and releases each
 * row (tcgen05.commit) once the last tile that reads it has been issued, and
 * two epilogue warpgroups (warps 0-3 and 4-7, alternating tiles; warp w reads
 * TMEM lanes 32 (w mod 4) ..) read an accumulator back with tcgen05.ld, apply
 * bias + ReLU (forward) or the ReLU mask of the layer input (data gradient)
 * and store bf16 NHWC.  Every mbarrier wait is bounded: on a timeout the CTA
 * raises a device status flag, drains its in-flight copies and MMAs (again
 * bounded), frees its tensor memory and returns.
 */
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "prml_internal.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int HC = 32;                     /* channels in and out */
constexpr int TM = 128;                    /* pixels per tile */
constexpr int SEG = TM + 2;                /* staged pixels per row */
constexpr int PIX_BYTES = HC * 2;          /* one staged pixel: 64 bytes */
constexpr unsigned TX_BYTES = SEG * PIX_BYTES; /* one staged row: 8320 bytes */
/* rows start on 1024-byte boundaries (the swizzle pattern repeats every 512) */
constexpr int ROW_BYTES = (int)((TX_BYTES + 1023) / 1024 * 1024);
constexpr int NROW = 8;                    /* staged-row ring (a power of two) */
constexpr int BAND = 16;                   /* output rows per work item */
constexpr int W_BYTES = 9 * 4 * HC * 16;   /* [tap][chunk][n][8] */
constexpr int NACC = 4;
constexpr int TMEM_COLS = 128;             /* NACC x 32 columns */
constexpr int EPI_GROUPS = 2;              /* epilogue warpgroups, alternating tiles */
constexpr int TMA_WARP = 4 * EPI_GROUPS, MMA_WARP = TMA_WARP + 1;
constexpr int THREADS = (MMA_WARP + 1) * 32;
static_assert(NACC % EPI_GROUPS == 0, "each group owns whole accumulators");
constexpr int BAR_BYTES = 256;
constexpr int SMEM_BYTES = NROW * ROW_BYTES + W_BYTES + BAR_BYTES + HC * 4 + 16 + 1024; /* + alignment slack */
constexpr unsigned long long kWaitNs = 2000000000ull; /* 2 s */
static_assert(ROW_BYTES % 1024 == 0, "swizzled TMA destinations start on 1024-byte boundaries");
static_assert((NROW * ROW_BYTES + W_BYTES) % 128 == 0, "weights and barriers aligned");
static_assert((2 * NROW + 2 * NACC) * 8 <= BAR_BYTES, "barrier area");
static_assert(NROW >= 4 && (NROW & (NROW - 1)) == 0, "ring of a power of two >= 4 rows");
static_assert((HC * 16 >> 4) < (1 << 14) && (512 >> 4) < (1 << 14), "descriptor offsets fit 14 bits");
static_assert(NROW * ROW_BYTES + W_BYTES < (1 << 18), "descriptor start fields (addr >> 4, 14 bits) never carry");

/* instruction descriptor, kind::f16: D f32, A bf16, B bf16, both K-major,
 * N = 32, M = 128 */
constexpr unsigned kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(HC >> 3) << 17) |
                            ((unsigned)(TM >> 4) << 24);

__device__ int g_cnn_tc_status;

__device__ __forceinline__ unsigned saddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void bar_init(unsigned long long* b, unsigned n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n) : "memory");
}

__device__ __forceinline__ bool bar_try(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

/* bounded wait; false after kWaitNs */
__device__ __forceinline__ bool bar_wait(unsigned long long* b, unsigned parity) {
  if (bar_try(b, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (!bar_try(b, parity))
    if (now_ns() - t0 > kWaitNs) return false;
  return true;
}

__device__ __forceinline__ void bar_arrive(unsigned long long* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}

__device__ __forceinline__ void bar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}

/* one staged row: box {32, 130, 1, 1} at (0, x, y, b), 64-byte swizzle */
__device__ __forceinline__ void tma_row(void* dst, const CUtensorMap* map, int x, int y, int b,
                                        unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cta.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(saddr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(0), "r"(x), "r"(y), "r"(b), "r"(saddr(bar))
      : "memory");
}

/* no-swizzle K-major shared memory descriptor */
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/* SWIZZLE_64B K-major descriptor (8-row groups 512 bytes apart).  The
 * swizzle follows the absolute shared-memory address bits, as the TMA
 * writes it, so a start shifted by whole pixels or by 32 bytes inside a row
 * needs no base offset (measured: base offset 0 matches the reference
 * convolution, the address-derived one does not). */
__device__ __forceinline__ unsigned long long smem_desc_sw64(unsigned addr) {
  return (unsigned long long)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((unsigned long long)(512u >> 4) << 32) |
         (1ull << 46) | (4ull << 61);
}

__device__ __forceinline__ void mma_f16(unsigned d_tmem, unsigned long long a, unsigned long long b,
                                        unsigned accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32]) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
      "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
      "[%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

struct Item {
  int b, r0, rows, x0;
};

/* work item t: image b, band of output rows [r0, r0 + rows), segment x0 */
__device__ __forceinline__ Item item_at(int t, int segs, int nbands, int H) {
  const int per_img = segs * nbands;
  Item it;
  it.b = t / per_img;
  const int r = t - it.b * per_img;
  const int band = r / segs;
  it.x0 = (r - band * segs) * TM;
  it.r0 = band * BAND;
  it.rows = H - it.r0 < BAND ? H - it.r0 : BAND;
  return it;
}

/* MODE 0: y = relu(conv(x, w) + bias).  MODE 1: y = conv(x, w) * (mask > 0).
 * w: [tap][n][k] bf16 (n = output channel). */
template <int MODE>
__global__ void __launch_bounds__(THREADS, 2) mid_conv_tc(const __grid_constant__ CUtensorMap xmap,
                                                          const bf16* __restrict__ w,
                                                          const float* __restrict__ bias,
                                                          const bf16* __restrict__ mask, bf16* __restrict__ y,
                                                          int B, int H, int W) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  unsigned char* rows = base;
  unsigned char* wsm = base + NROW * ROW_BYTES;
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(wsm + W_BYTES);
  unsigned long long* full = bars;                 /* [NROW] */
  unsigned long long* empty = bars + NROW;         /* [NROW] */
  unsigned long long* accfull = bars + 2 * NROW;   /* [NACC] */
  unsigned long long* accempty = accfull + NACC;   /* [NACC] */
  float* bias_s = reinterpret_cast<float*>(wsm + W_BYTES + BAR_BYTES);
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(bias_s + HC);
  __shared__ int abort_flag;
  __shared__ int loads_issued;  /* row loads issued by the producer */
  __shared__ int loads_waited;  /* row loads the MMA warp has seen land */
  __shared__ int tiles_issued;  /* tiles whose MMAs were issued */

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int segs = (W + TM - 1) / TM;
  const int nbands = (H + BAND - 1) / BAND;
  const int items = B * segs * nbands;

  /* weights [tap][n][k] -> [tap][chunk][n][8], bias */
  for (int i = tid; i < 9 * HC * 4; i += THREADS) {
    const int tap = i / (HC * 4), rem = i - tap * HC * 4, n = rem >> 2, c = rem & 3;
    const uint4 v = *reinterpret_cast<const uint4*>(w + (tap * HC + n) * HC + c * 8);
    *reinterpret_cast<uint4*>(wsm + ((tap * 4 + c) * HC + n) * 16) = v;
  }
  if (MODE == 0 && tid < HC) bias_s[tid] = bias[tid];
  if (tid == 0) {
    for (int s = 0; s < NROW; ++s) {
      bar_init(&full[s], 1);
      bar_init(&empty[s], 1);
    }
    for (int a = 0; a < NACC; ++a) {
      bar_init(&accfull[a], 1);
      bar_init(&accempty[a], 4 * 32);
    }
    abort_flag = 0;
    loads_issued = 0;
    loads_waited = 0;
    tiles_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  /* generic-proxy weight stores must be visible to the tensor cores */
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *tmem_slot;

  if (warp == TMA_WARP) {
    /* ---- row loads */
    if (lane == 0) {
      int L = 0;
      for (int t = blockIdx.x; t < items && !abort_flag; t += gridDim.x) {
        const Item it = item_at(t, segs, nbands, H);
        for (int j = 0; j < it.rows + 2; ++j, ++L) {
          const int q = L % NROW;
          unsigned char* dst = rows + q * ROW_BYTES;
          if (!bar_wait(&empty[q], ((L / NROW) & 1) ^ 1) || *(volatile int*)&abort_flag ||
              (saddr(dst) & 1023u)) { /* the last test: never issue a misaligned copy */
            atomicExch(&abort_flag, 1);
            break;
          }
          bar_expect_tx(&full[q], TX_BYTES);
          tma_row(dst, &xmap, it.x0 - 1, it.r0 - 1 + j, it.b, &full[q]);
          loads_issued = L + 1;
        }
      }
    }
  } else if (warp == MMA_WARP) {
    /* ---- MMA issuer */
    if (lane == 0) {
      const unsigned wbase = saddr(wsm);
      int L0 = 0, T = 0;
      bool ok = (wbase & 15u) == 0;
      /* ring rows are ROW_BYTES apart: slot q's descriptor is adesc0 + q * (ROW_BYTES >> 4) */
      const unsigned long long adesc0 = smem_desc_sw64(saddr(rows));
      const unsigned long long bdesc = smem_desc(wbase, HC * 16, 128);
      auto adesc = [&](int L) {
        return adesc0 + (unsigned long long)((L & (NROW - 1)) * (ROW_BYTES >> 4));
      };
      auto landed = [&](int L) {
        if (!bar_wait(&full[L % NROW], (L / NROW) & 1)) return false;
        loads_waited = L + 1;
        return true;
      };
      for (int t = blockIdx.x; t < items && ok; t += gridDim.x) {
        const Item it = item_at(t, segs, nbands, H);
        ok = landed(L0) && landed(L0 + 1);
        for (int i = 0; i < it.rows && ok; ++i, ++T) {
          const int a = T % NACC;
          ok = landed(L0 + i + 2) && bar_wait(&accempty[a], ((T / NACC) & 1) ^ 1) &&
               !*(volatile int*)&abort_flag;
          if (!ok) break;
          tc_fence_after();
          const unsigned d = tmem + (unsigned)(a * HC);
          /* descriptors are linear in the start address (field = addr >> 4,
           * no carry for shared addresses), so each MMA's operands are a
           * constant add to the base descriptor of its row slot / weights */
          const unsigned long long r0 = adesc(L0 + i);
          const unsigned long long r1 = adesc(L0 + i + 1);
          const unsigned long long r2 = adesc(L0 + i + 2);
#pragma unroll
          for (int tap = 0; tap < 9; ++tap) {
            const unsigned long long ra = tap < 3 ? r0 : (tap < 6 ? r1 : r2);
#pragma unroll
            for (int kk = 0; kk < 2; ++kk)
              mma_f16(d, ra + (unsigned long long)(((tap % 3) * PIX_BYTES + kk * 32) >> 4),
                      bdesc + (unsigned long long)(((tap * 4 + 2 * kk) * HC * 16) >> 4),
                      (tap > 0 || kk > 0) ? 1u : 0u);
          }
          mma_commit(&accfull[a]);                /* the accumulator is ready */
          mma_commit(&empty[(L0 + i) % NROW]);    /* row y-1 is read for the last time */
          tiles_issued = T + 1;
        }
        if (!ok) break;
        /* the band's last two rows are free once its last MMAs are done */
        mma_commit(&empty[(L0 + it.rows) % NROW]);
        mma_commit(&empty[(L0 + it.rows + 1) % NROW]);
        L0 += it.rows + 2;
      }
      if (!ok) atomicExch(&abort_flag, 1);
    }
  } else {
    /* ---- epilogue: group g takes the tiles T with T mod EPI_GROUPS == g;
     * warp w owns TMEM lanes 32 (w mod 4) .. = tile pixels */
    const int group = warp >> 2, wq = warp & 3;
    int T = 0;
    bool go = true;
    for (int t = blockIdx.x; t < items && go; t += gridDim.x) {
      const Item it = item_at(t, segs, nbands, H);
      for (int i = 0; i < it.rows; ++i, ++T) {
        if (T % EPI_GROUPS != group) continue;
        const int a = T % NACC;
        const bool ok = bar_wait(&accfull[a], (T / NACC) & 1);
        if (__any_sync(0xffffffffu, !ok) || *(volatile int*)&abort_flag) {
          atomicExch(&abort_flag, 1);
          go = false;
          break;
        }
        tc_fence_after();
        float v[32];
        tmem_ld32(tmem + ((unsigned)(wq * 32) << 16) + (unsigned)(a * HC), v);
        tc_fence_before();
        bar_arrive(&accempty[a]);
        const int gx = it.x0 + wq * 32 + lane;
        if (gx < W) {
          const long long p = ((long long)it.b * H + it.r0 + i) * W + gx;
          if (MODE == 0) {
#pragma unroll
            for (int k = 0; k < 32; ++k) v[k] = fmaxf(v[k] + bias_s[k], 0.f);
          } else {
            const uint4* mp = reinterpret_cast<const uint4*>(mask + p * HC);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const uint4 m = mp[q];
              const __nv_bfloat162* mh = reinterpret_cast<const __nv_bfloat162*>(&m);
#pragma unroll
              for (int j = 0; j < 4; ++j) {
                const float2 f = __bfloat1622float2(mh[j]);
                if (!(f.x > 0.f)) v[q * 8 + 2 * j] = 0.f;
                if (!(f.y > 0.f)) v[q * 8 + 2 * j + 1] = 0.f;
              }
            }
          }
          uint4* yp = reinterpret_cast<uint4*>(y + p * HC);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            uint4 o;
            __nv_bfloat162* oh = reinterpret_cast<__nv_bfloat162*>(&o);
#pragma unroll
            for (int j = 0; j < 4; ++j) oh[j] = __floats2bfloat162_rn(v[q * 8 + 2 * j], v[q * 8 + 2 * j + 1]);
            yp[q] = o;
          }
        }
      }
    }
  }

  /* ---- drain (bounded) and free tensor memory */
  __syncthreads();
  if (abort_flag) {
    if (tid == 0) atomicExch(&g_cnn_tc_status, 1);
    if (warp == TMA_WARP && lane == 0) {
      /* row loads issued but never seen by the MMA warp */
      for (int j = loads_waited; j < loads_issued; ++j) bar_wait(&full[j % NROW], (j / NROW) & 1);
    }
    if (warp == MMA_WARP && lane == 0 && tiles_issued > 0) {
      const int j = tiles_issued - 1;
      bar_wait(&accfull[j % NACC], (j / NACC) & 1);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

/* ---- weight gradient of the 32 -> 32 convolutions ---------------------------
 * dW[dy][dx][co][ci] = sum over pixels p of g[p][co] x[p + (dy - 1, dx - 1)][ci]
 * (x zero outside the image) as tcgen05 MMAs whose K is pixels.  D (M = 128,
 * N = 32, f32 in TMEM) row 32 j + ci holds the column shift j - 1 of input
 * channel ci for every output channel; j = 3 (a shift of +2) is computed and
 * discarded, so one MMA covers a kernel row's three taps.  One accumulator
 * per kernel row dy (96 TMEM columns).  Both operands are the staged NHWC
 * rows read MN-major with the 64-byte swizzle (a pixel's 32 channels are one
 * 64-byte row of a swizzle atom, 8 pixels one 512-byte atom): A = the input
 * row y + dy - 1 from one pixel left of the K block, its four 32-row MN
 * blocks one pixel (64 bytes, the leading byte offset) apart, 8-pixel K
 * groups 512 bytes (the stride byte offset) apart; B = the gradient row y.
 * A CTA walks (image, band, 128-pixel segment) items as the convolution does,
 * accumulates over all of them, and writes its partial dW [tap][co][ci]
 * once at the end.  Roles: warp 4 loads rows (input rows through the ring of
 * NROW, gradient rows through a ring of WG_NG), warp 5 issues the MMAs,
 * warps 0-3 read the accumulators back.  Waits are bounded as in the
 * convolution. */
constexpr int WG_G_BYTES = TM * PIX_BYTES; /* one gradient row, 8192 bytes */
constexpr int WG_NG = 4;
constexpr int WG_TMEM_COLS = 128;          /* 3 x 32 used */
constexpr int WG_TMA_WARP = 4, WG_MMA_WARP = 5;
constexpr int WG_THREADS = 6 * 32;
/* + alignment slack + room for reads of the discarded shift past a row */
constexpr int WG_SMEM = NROW * ROW_BYTES + WG_NG * WG_G_BYTES + BAR_BYTES + 1024 + 2048;
constexpr unsigned kIdescWg = kIdesc | (1u << 15) | (1u << 16); /* A and B MN-major */
static_assert(WG_G_BYTES % 1024 == 0, "gradient rows start on 1024-byte boundaries");
static_assert((2 * NROW + 2 * WG_NG + 1) * 8 <= BAR_BYTES, "barrier area");
static_assert(NROW * ROW_BYTES + WG_NG * WG_G_BYTES + BAR_BYTES < (1 << 18), "descriptor start fields never carry");

/* SWIZZLE_64B MN-major descriptor: MN blocks of 32 elements `lbo` bytes
 * apart, 8-row K groups 512 bytes apart */
__device__ __forceinline__ unsigned long long smem_desc_mn_sw64(unsigned addr, unsigned lbo) {
  return (unsigned long long)((addr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)(512u >> 4) << 32) | (1ull << 46) | (4ull << 61);
}

__device__ __forceinline__ void mma_f16_wg(unsigned d_tmem, unsigned long long a, unsigned long long b,
                                           unsigned accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdescWg), "r"(accumulate)
      : "memory");
}

/* one gradient row: box {32, 128, 1, 1} at (0, x, y, b), 64-byte swizzle */
__device__ __forceinline__ void tma_grow(void* dst, const CUtensorMap* map, int x, int y, int b,
                                         unsigned long long* bar) {
  tma_row(dst, map, x, y, b, bar);
}

__global__ void __launch_bounds__(WG_THREADS, 2) mid_wgrad_tc(const __grid_constant__ CUtensorMap xmap,
                                                              const __grid_constant__ CUtensorMap gmap,
                                                              float* __restrict__ partial, int B, int H, int W) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
  unsigned char* xrows = base;
  unsigned char* grows = base + NROW * ROW_BYTES;
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(grows + WG_NG * WG_G_BYTES);
  unsigned long long* xfull = bars;                  /* [NROW] */
  unsigned long long* xempty = bars + NROW;          /* [NROW] */
  unsigned long long* gfull = bars + 2 * NROW;       /* [WG_NG] */
  unsigned long long* gempty = gfull + WG_NG;        /* [WG_NG] */
  unsigned long long* done = gempty + WG_NG;         /* all MMAs complete */
  __shared__ unsigned tmem_slot;
  __shared__ int abort_flag;
  __shared__ int xl_issued, xl_waited, gl_issued, gl_waited;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int segs = (W + TM - 1) / TM;
  const int nbands = (H + BAND - 1) / BAND;
  const int items = B * segs * nbands;

  if (tid == 0) {
    for (int q = 0; q < NROW; ++q) {
      bar_init(&xfull[q], 1);
      bar_init(&xempty[q], 1);
    }
    for (int q = 0; q < WG_NG; ++q) {
      bar_init(&gfull[q], 1);
      bar_init(&gempty[q], 1);
    }
    bar_init(done, 1);
    abort_flag = 0;
    xl_issued = xl_waited = gl_issued = gl_waited = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tmem_slot)),
                 "r"(WG_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = tmem_slot;

  if (warp == WG_TMA_WARP) {
    /* ---- row loads: input rows r0 - 1 .. r0 + rows, and after input row
     * j the gradient row j - 2 (so an output row's inputs arrive together) */
    if (lane == 0) {
      int L = 0, G = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < items && ok; t += gridDim.x) {
        const Item it = item_at(t, segs, nbands, H);
        for (int j = 0; j < it.rows + 2 && ok; ++j) {
          const int q = L % NROW;
          unsigned char* dst = xrows + q * ROW_BYTES;
          ok = bar_wait(&xempty[q], ((L / NROW) & 1) ^ 1) && !*(volatile int*)&abort_flag &&
               (saddr(dst) & 1023u) == 0;
          if (!ok) break;
          bar_expect_tx(&xfull[q], TX_BYTES);
          tma_row(dst, &xmap, it.x0 - 1, it.r0 - 1 + j, it.b, &xfull[q]);
          xl_issued = ++L;
          if (j >= 2) {
            const int qg = G % WG_NG;
            unsigned char* gdst = grows + qg * WG_G_BYTES;
            ok = bar_wait(&gempty[qg], ((G / WG_NG) & 1) ^ 1) && !*(volatile int*)&abort_flag &&
                 (saddr(gdst) & 1023u) == 0;
            if (!ok) break;
            bar_expect_tx(&gfull[qg], WG_G_BYTES);
            tma_grow(gdst, &gmap, it.x0, it.r0 + j - 2, it.b, &gfull[qg]);
            gl_issued = ++G;
          }
        }
      }
      if (!ok) atomicExch(&abort_flag, 1);
    }
  } else if (warp == WG_MMA_WARP) {
    /* ---- MMA issuer */
    if (lane == 0) {
      int L0 = 0, G0 = 0, T = 0;
      bool ok = true;
      auto xlanded = [&](int L) {
        if (!bar_wait(&xfull[L % NROW], (L / NROW) & 1)) return false;
        xl_waited = L + 1;
        return true;
      };
      const unsigned xbase = saddr(xrows), gbase = saddr(grows);
      for (int t = blockIdx.x; t < items && ok; t += gridDim.x) {
        const Item it = item_at(t, segs, nbands, H);
        /* K blocks holding pixels of the image: past it the gradient is
         * zero (the last segment of a 257-wide row holds one pixel) */
        const int ksteps = (W - it.x0 >= TM) ? TM / 16 : (W - it.x0 + 15) / 16;
        ok = xlanded(L0) && xlanded(L0 + 1);
        for (int i = 0; i < it.rows && ok; ++i, ++T) {
          const int qg = (G0 + i) % WG_NG;
          ok = xlanded(L0 + i + 2) && bar_wait(&gfull[qg], ((G0 + i) / WG_NG) & 1) &&
               !*(volatile int*)&abort_flag;
          if (!ok) break;
          gl_waited = G0 + i + 1;
          tc_fence_after();
#pragma unroll
          for (int dy = 0; dy < 3; ++dy) {
            const unsigned xr = xbase + (unsigned)(((L0 + i + dy) % NROW) * ROW_BYTES);
            const unsigned gr = gbase + (unsigned)(qg * WG_G_BYTES);
            for (int k = 0; k < ksteps; ++k)
              mma_f16_wg(tmem + (unsigned)(dy * HC), smem_desc_mn_sw64(xr + (unsigned)(k * 16 * PIX_BYTES), PIX_BYTES),
                         smem_desc_mn_sw64(gr + (unsigned)(k * 16 * PIX_BYTES), PIX_BYTES),
                         (T > 0 || k > 0) ? 1u : 0u);
          }
          mma_commit(&xempty[(L0 + i) % NROW]);  /* input row y - 1 is read for the last time */
          mma_commit(&gempty[qg]);
        }
        if (!ok) break;
        mma_commit(&xempty[(L0 + it.rows) % NROW]);
        mma_commit(&xempty[(L0 + it.rows + 1) % NROW]);
        L0 += it.rows + 2;
        G0 += it.rows;
      }
      if (!ok) atomicExch(&abort_flag, 1);
      mma_commit(done); /* arrives once every MMA issued above has completed */
    }
  } else {
    /* ---- epilogue: warp w reads TMEM lanes 32 w .. (shift j = w, channel
     * ci = lane) of each kernel row's accumulator */
    const bool ok = bar_wait(done, 0);
    if (__any_sync(0xffffffffu, !ok)) atomicExch(&abort_flag, 1);
    if (ok && !*(volatile int*)&abort_flag && warp < 3) {
      /* the grid never exceeds the items, so every CTA accumulated rows */
      float* out = partial + (long long)blockIdx.x * 9 * HC * HC;
#pragma unroll
      for (int dy = 0; dy < 3; ++dy) {
        float v[32];
        tc_fence_after();
        tmem_ld32(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)(dy * HC), v);
        const int tap = dy * 3 + warp;
#pragma unroll
        for (int co = 0; co < HC; ++co) out[(tap * HC + co) * HC + lane] = v[co];
      }
    }
  }

  /* ---- drain (bounded) and free tensor memory */
  __syncthreads();
  if (abort_flag) {
    if (tid == 0) atomicExch(&g_cnn_tc_status, 1);
    if (warp == WG_TMA_WARP && lane == 0) {
      for (int j = xl_waited; j < xl_issued; ++j) bar_wait(&xfull[j % NROW], (j / NROW) & 1);
      for (int j = gl_waited; j < gl_issued; ++j) bar_wait(&gfull[j % WG_NG], (j / WG_NG) & 1);
    }
    if (warp == WG_MMA_WARP && lane == 0) bar_wait(done, 0);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(WG_TMEM_COLS) : "memory");
}

int g_tc_path = 1;

template <int MODE>
int launch(const void* x, const void* w, const float* bias, const void* mask, void* y, int B, int H, int W,
           void* stream) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(mid_conv_tc<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("mid_conv_tc attribute: ") + cudaGetErrorString(e));
    attr_set = true;
  }
  if ((reinterpret_cast<unsigned long long>(x) & 15ull) || (reinterpret_cast<unsigned long long>(w) & 15ull) ||
      (reinterpret_cast<unsigned long long>(y) & 15ull) || (mask && (reinterpret_cast<unsigned long long>(mask) & 15ull)))
    return prml_set_error(PRML_ERR_ARG, "mid_conv_tc: buffers must be 16-byte aligned");
  /* x as [B][H][W][32]: dims innermost first */
  const unsigned long long dims[4] = {32, (unsigned long long)W, (unsigned long long)H, (unsigned long long)B};
  const unsigned long long strides[3] = {64, 64ull * W, 64ull * W * H};
  const unsigned box[4] = {32, SEG, 1, 1};
  CUtensorMap map;
  int rc = prml_tensor_map_tiled(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, x, dims, strides, box, 64);
  if (rc) return rc;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long items = (long long)B * ((H + BAND - 1) / BAND) * ((W + TM - 1) / TM);
  if (items > 0x7fffffffLL) return prml_set_error(PRML_ERR_ARG, "mid_conv_tc: too many work items");
  const int grid = (int)(items < 2LL * sms ? items : 2LL * sms);
  mid_conv_tc<MODE><<<grid, THREADS, SMEM_BYTES, static_cast<cudaStream_t>(stream)>>>(
      map, static_cast<const bf16*>(w), bias, static_cast<const bf16*>(mask), static_cast<bf16*>(y), B, H, W);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("mid_conv_tc: ") + cudaGetErrorString(e));
  return PRML_OK;
}

int launch_wgrad(const void* x, const void* g, float* partial, int parts, int* used, int B, int H, int W,
                 void* stream) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(mid_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, WG_SMEM);
    if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("mid_wgrad_tc attribute: ") + cudaGetErrorString(e));
    attr_set = true;
  }
  if ((reinterpret_cast<unsigned long long>(x) & 15ull) || (reinterpret_cast<unsigned long long>(g) & 15ull))
    return prml_set_error(PRML_ERR_ARG, "mid_wgrad_tc: buffers must be 16-byte aligned");
  const unsigned long long dims[4] = {32, (unsigned long long)W, (unsigned long long)H, (unsigned long long)B};
  const unsigned long long strides[3] = {64, 64ull * W, 64ull * W * H};
  const unsigned xbox[4] = {32, SEG, 1, 1};
  const unsigned gbox[4] = {32, TM, 1, 1};
  CUtensorMap xmap, gmap;
  int rc = prml_tensor_map_tiled(&xmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, x, dims, strides, xbox, 64);
  if (rc) return rc;
  rc = prml_tensor_map_tiled(&gmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, g, dims, strides, gbox, 64);
  if (rc) return rc;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long items = (long long)B * ((H + BAND - 1) / BAND) * ((W + TM - 1) / TM);
  if (items > 0x7fffffffLL) return prml_set_error(PRML_ERR_ARG, "mid_wgrad_tc: too many work items");
  long long grid = 2LL * sms;
  if (grid > parts) grid = parts;
  if (grid > items) grid = items;
  *used = (int)grid;
  mid_wgrad_tc<<<(int)grid, WG_THREADS, WG_SMEM, static_cast<cudaStream_t>(stream)>>>(xmap, gmap, partial, B, H, W);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("mid_wgrad_tc: ") + cudaGetErrorString(e));
  return PRML_OK;
}

}  // namespace

int prml_cnn_tc_enabled() { return g_tc_path; }

int prml_cnn_mid_wgrad_tc(const void* x, const void* g, float* partial, int parts, int* used, int B, int H, int W,
                          void* stream) {
  return launch_wgrad(x, g, partial, parts, used, B, H, W, stream);
}

int prml_cnn_mid_conv_tc(int mode, const void* x, const void* w, const float* bias, const void* mask, void* y,
                         int B, int H, int W, void* stream) {
  return mode == 0 ? launch<0>(x, w, bias, mask, y, B, H, W, stream)
                   : launch<1>(x, w, bias, mask, y, B, H, W, stream);
}

extern "C" {

int prml_cnn_set_tensor_path(int tcgen05) {
  const int prev = g_tc_path;
  g_tc_path = tcgen05 ? 1 : 0;
  return prev;
}

int prml_cnn_status(void) {
  int flag = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&flag, g_cnn_tc_status, sizeof(int));
  if (e != cudaSuccess) return prml_set_error(PRML_ERR_CUDA, std::string("prml_cnn_status: ") + cudaGetErrorString(e));
  if (flag) {
    const int zero = 0;
    cudaMemcpyToSymbol(g_cnn_tc_status, &zero, sizeof(int));
    return prml_set_error(PRML_ERR_CUDA, "a tensor-core convolution timed out waiting on its pipeline");
  }
  return PRML_OK;
}

}  // extern "C"
