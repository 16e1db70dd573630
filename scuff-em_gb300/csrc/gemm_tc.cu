// gemm_tc.cu -- tensor-core trailing update of the complex-FP32 LU:
//     C (m x n, complex64, column-major) -= A (m x k) * B (k x n)
// on sm_103a with tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulators in
// tensor memory), TMA tile loads into 128B-swizzled shared memory and
// mbarrier-tracked pipelining.
//
// Complex FP32 accuracy from BF16 tensor cores (the "split-BF16" form):
// each FP32 value x is split into hi = bf16(x) and lo = bf16(x - hi), and
// A B ~= Ah Bh + Ah Bl + Al Bh.  Together with the real embedding of the
// complex product,
//     [Re C | Im C] = [Ar | Ai] x [[Br, Bi], [-Bi, Br]],
// the whole update is ONE real GEMM with K'' = 3 * 2k:
//     Ahat (m x 6k)   row i   = [Ar_h Ai_h | Ar_h Ai_h | Ar_l Ai_l]
//     Bhat (2n x 6k)  row 2j  = [Br_h -Bi_h | Br_l -Bi_l | Br_h -Bi_h]
//                     row 2j+1= [Bi_h  Br_h | Bi_l  Br_l | Bi_h  Br_h]
// whose output columns (2j, 2j+1) are exactly (Re, Im) of C[:, j], so the
// epilogue writes interleaved complex64 with coalesced stores.
//
// Kernel layout (one CTA per 128 x 256 output tile, 10 warps):
//   warp 0   TMA producer (one elected lane), 4-stage ring of (A 16 KB, B 32 KB)
//   warp 1   TMEM allocator and MMA issuer (one lane): 4 x (M128 N256 K16)
//            per 64-wide k-block, tcgen05.commit frees the stage
//   warps 2-9 epilogue: tcgen05.ld 32 lanes x 32 columns at a time, C -= D
//            (C loads issued before the TMEM read so they overlap)
// Every mbarrier wait is bounded; on timeout the CTA records an error code,
// drains its outstanding TMA copies (bounded), frees its TMEM and exits.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include "bem_math.cuh"
#include "gbem_internal.h"

namespace gbem {

namespace tc {
constexpr int BM = 128, BN = 256, BK = 64, STAGES = 4;
constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
static_assert((2 * STAGES + 5) * 8 + 4 <= 256, "barrier area");
constexpr uint32_t TMEM_COLS = 256;
constexpr long long SPIN_LIMIT = 1ll << 20;  // bounded waits (about a second at most)
}  // namespace tc

__device__ int g_tc_error = 0;

// ---------------- PTX helpers ----------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long it = 0; it < tc::SPIN_LIMIT; it++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)(16 >> 4) << 16;    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;            // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

// instruction descriptor: D f32, A/B bf16, both K-major, M = 128, N = 256
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(tc::BN >> 3) << 17) |
                           ((uint32_t)(tc::BM >> 4) << 24);

__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// ---------------- split packing ----------------
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16* hi, __nv_bfloat16* lo) {
  __nv_bfloat16 h = __float2bfloat16_rn(x);
  *hi = h;
  *lo = __float2bfloat16_rn(x - __bfloat162float(h));
}

// Ahat rows, 16 rows per CTA (k <= 256): the rows' k complex values are staged
// in shared memory by coalesced column reads, then each row (Kp bf16, zero
// padded past 6k) is written with contiguous 8-byte stores.
__global__ void __launch_bounds__(256) pack_a(const cx<float>* A, long long lda, int m, int k, int Kp,
                                              __nv_bfloat16* out) {
  pdl_wait();
  pdl_trigger();
  __shared__ cx<float> t[256][17];
  const int i0 = blockIdx.x * 16;
  for (int q = threadIdx.x; q < 16 * k; q += blockDim.x) {
    const int r = q & 15, kk = q >> 4, i = i0 + r;
    t[kk][r] = i < m ? A[i + (long long)kk * lda] : mk(0.0f, 0.0f);
  }
  __syncthreads();
  const int words = Kp >> 2;  // 4 bf16 per 8-byte store
  for (int q = threadIdx.x; q < 16 * words; q += blockDim.x) {
    const int r = q / words, w4 = q - r * words, i = i0 + r;
    if (i >= m) continue;
    __nv_bfloat16 v[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int p = 4 * w4 + e, seg = p / k, kk = p - seg * k;
      float x = 0.0f;
      bool lo = false;
      if (seg < 6) {
        const cx<float> z = t[kk][r];
        x = (seg & 1) ? z.im : z.re;
        lo = seg >= 4;
      }
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      v[e] = lo ? __float2bfloat16_rn(x - __bfloat162float(h)) : h;
    }
    uint2 pk;
    pk.x = (uint32_t)__bfloat16_as_ushort(v[0]) | ((uint32_t)__bfloat16_as_ushort(v[1]) << 16);
    pk.y = (uint32_t)__bfloat16_as_ushort(v[2]) | ((uint32_t)__bfloat16_as_ushort(v[3]) << 16);
    *reinterpret_cast<uint2*>(out + (long long)i * Kp + 4 * w4) = pk;
  }
}

__global__ void pack_b(const cx<float>* B, long long ldb, int k, int n, int Kp, __nv_bfloat16* out) {
  pdl_wait();
  pdl_trigger();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)k * n) return;
  int kk = (int)(t % k), j = (int)(t / k);
  cx<float> b = B[kk + (long long)j * ldb];
  __nv_bfloat16 rh, rl, ih, il;
  split_bf16(b.re, &rh, &rl);
  split_bf16(b.im, &ih, &il);
  __nv_bfloat16 nih = __hneg(ih), nil = __hneg(il);
  __nv_bfloat16* r0 = out + (long long)(2 * j) * Kp;
  __nv_bfloat16* r1 = r0 + Kp;
  r0[kk] = rh; r0[k + kk] = nih; r0[2 * k + kk] = rl; r0[3 * k + kk] = nil; r0[4 * k + kk] = rh; r0[5 * k + kk] = nih;
  r1[kk] = ih; r1[k + kk] = rh;  r1[2 * k + kk] = il; r1[3 * k + kk] = rl;  r1[4 * k + kk] = ih; r1[5 * k + kk] = rh;
}

__global__ void zero_pad(__nv_bfloat16* out, long long rows, int K6, int Kp) {
  pdl_wait();
  pdl_trigger();
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int w = Kp - K6;
  if (w <= 0 || t >= rows * w) return;
  out[(t / w) * Kp + K6 + (t % w)] = __float2bfloat16_rn(0.0f);
}

// ---------------- the GEMM kernel ----------------
// Persistent: CTA c takes output tiles c, c + P, c + 2P, ... (P = gridDim.x;
// tiles ordered with the m index fastest, so the CTAs of a wave share their B
// tile).  Two 256-column accumulators in TMEM: the MMAs of tile i+1 run while
// the epilogue warps drain tile i.
__global__ void __launch_bounds__(320, 1) tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA,
                                                          const __grid_constant__ CUtensorMap mapB, cx<float>* C,
                                                          long long ldc, int m, int n, int kblocks, int mt,
                                                          int ntiles) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  uintptr_t base = ((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023;
  unsigned char* tiles = (unsigned char*)base;
  uint64_t* full = (uint64_t*)(tiles + tc::STAGES * tc::STAGE_BYTES);
  uint64_t* empty = full + tc::STAGES;
  uint64_t* acc_full = empty + tc::STAGES;  // [2] MMA -> epilogue
  uint64_t* acc_empty = acc_full + 2;       // [2] epilogue -> MMA (8 warp arrivals)
  uint64_t* drain = acc_empty + 2;          // all MMAs retired
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // once any CTA has given up on a wait, the rest of the grid does no work
  if (*(volatile int*)&g_tc_error) return;

  if (threadIdx.x == 0) {
    for (int s = 0; s < tc::STAGES; s++) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    for (int a = 0; a < 2; a++) { mbar_init(&acc_full[a], 1); mbar_init(&acc_empty[a], 8); }
    mbar_init(drain, 1);
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * tc::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // producer: one ring of STAGES slots across all of this CTA's tiles
      long long g = 0, issued = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int tm = t % mt, tn = t / mt;
        for (int kb = 0; kb < kblocks; kb++, g++) {
          const int s = (int)(g % tc::STAGES);
          if (g >= tc::STAGES) {
            if (!mbar_wait(&empty[s], (uint32_t)(((g / tc::STAGES) - 1) & 1))) { atomicExch(&s_fail, 1); ok = false; break; }
          }
          unsigned char* sa = tiles + s * tc::STAGE_BYTES;
          mbar_arrive_expect_tx(&full[s], tc::STAGE_BYTES);
          tma_load_2d(sa, &mapA, &full[s], kb * tc::BK, tm * tc::BM);
          tma_load_2d(sa + tc::A_BYTES, &mapB, &full[s], kb * tc::BK, tn * tc::BN);
          issued = g + 1;
        }
      }
      // drain: no TMA write may still be in flight when the CTA exits
      for (long long q = (issued > tc::STAGES ? issued - tc::STAGES : 0); q < issued; q++)
        mbar_wait(&full[q % tc::STAGES], (uint32_t)((q / tc::STAGES) & 1));
    }
  } else if (warp == 1) {
    if (lane == 0) {
      long long g = 0;
      bool ok = true;
      int i = 0;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, i++) {
        const int acc = i & 1;
        if (i >= 2 && !mbar_wait(&acc_empty[acc], (uint32_t)(((i >> 1) - 1) & 1))) {
          atomicExch(&s_fail, 1);
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(acc * tc::TMEM_COLS);
        for (int kb = 0; kb < kblocks; kb++, g++) {
          const int s = (int)(g % tc::STAGES);
          if (!mbar_wait(&full[s], (uint32_t)((g / tc::STAGES) & 1))) { atomicExch(&s_fail, 1); ok = false; break; }
          tc_fence_after();
          uint32_t a0 = smem_u32(tiles + s * tc::STAGE_BYTES), b0 = a0 + tc::A_BYTES;
          for (int kk = 0; kk < tc::BK / 16; kk++) {
            uint64_t da = sdesc_sw128(a0 + kk * 32), db = sdesc_sw128(b0 + kk * 32);
            umma_f16(d, da, db, (kb > 0 || kk > 0) ? 1u : 0u);
          }
          umma_commit(&empty[s]);
        }
        if (ok) umma_commit(&acc_full[acc]);
      }
      // every MMA issued so far has retired once this barrier completes
      umma_commit(drain);
      if (!mbar_wait(drain, 0)) atomicExch(&s_fail, 1);
    }
  } else {
    // epilogue warps 2..9: warp % 4 selects the TMEM lane quarter (row block
    // of 32), the two warps of a quarter split the 256 accumulator columns
    const int q = warp & 3, half = (warp - 2) >> 2;
    int i = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
      const int acc = i & 1;
      const int tm = t % mt, tn = t / mt;
      const int row = tm * tc::BM + q * 32 + lane;
      const bool ok = mbar_wait(&acc_full[acc], (uint32_t)((i >> 1) & 1));
      if (!ok) atomicExch(&s_fail, 1);
      if (!ok || *(volatile int*)&s_fail) break;
      tc_fence_after();
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * tc::TMEM_COLS);
      for (int c0 = half * (tc::BN / 2); c0 < (half + 1) * (tc::BN / 2); c0 += 32) {
        const int j0 = (tn * tc::BN + c0) >> 1;
        // issue the 16 loads of C first (independent), then the TMEM read
        cx<float> z[16];
#pragma unroll
        for (int u = 0; u < 16; u++)
          z[u] = (row < m && j0 + u < n) ? C[row + (long long)(j0 + u) * ldc] : mk(0.0f, 0.0f);
        float v[32];
        tmem_ld32(tbase + (uint32_t)c0, v);
        if (c0 + 32 >= (half + 1) * (tc::BN / 2)) {
          // last TMEM read of this warp for the tile: hand the accumulator back
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&acc_empty[acc]);
        }
#pragma unroll
        for (int u = 0; u < 16; u++) {
          if (row < m && j0 + u < n) {
            z[u].re -= v[2 * u];
            z[u].im -= v[2 * u + 1];
            C[row + (long long)(j0 + u) * ldc] = z[u];
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * tc::TMEM_COLS));
  }
  if (threadIdx.x == 0 && s_fail) atomicExch(&g_tc_error, 1);
}

// ---------------- host side ----------------
static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

static bool make_map(CUtensorMap* map, const void* ptr, int rows, int Kp, int box_rows) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

static int pad64(int x) { return (x + 63) / 64 * 64; }

size_t tc_gemm_ws_bytes(int m, int n, int k) {
  size_t Kp = (size_t)pad64(6 * k);
  return ((size_t)m + 2 * (size_t)n) * Kp * 2 + 4096;
}

static int g_tc_mode = -1;  // -1 unknown, 0 disabled, 1 enabled
static thread_local int tl_tc_off = 0;  // this host thread's LU takes the FP32 SIMT updates

void tc_gemm_set_enabled(int on) { g_tc_mode = on ? 1 : 0; }
void tc_gemm_thread_off(int off) { tl_tc_off = off; }

bool tc_gemm_update(cx<float>* C, long long ldc, const cx<float>* A, long long lda, const cx<float>* B, long long ldb,
                    int m, int n, int k, void* ws, size_t ws_bytes, cudaStream_t s, cudaError_t* err) {
  *err = cudaSuccess;
  if (g_tc_mode < 0) {
    const char* e = getenv("GBEM_LU_TC");
    g_tc_mode = (e && e[0] == '0') ? 0 : 1;
  }
  if (g_tc_mode == 0 || tl_tc_off) return false;
  if (m <= 0 || n <= 0 || k <= 0) return true;
  int Kp = pad64(6 * k);
  size_t need = ((size_t)m + 2 * (size_t)n) * Kp * 2;
  if (!ws || ws_bytes < need) return false;
  __nv_bfloat16* pa = (__nv_bfloat16*)ws;
  __nv_bfloat16* pb = pa + (size_t)m * Kp;
  if (k > 256) return false;
  long long tb = (long long)k * n;
  launch_pdl(pack_a, dim3((unsigned)((m + 15) / 16)), dim3(256), 0, s, A, lda, m, k, Kp, pa);
  launch_pdl(pack_b, dim3((unsigned)((tb + 255) / 256)), dim3(256), 0, s, B, ldb, k, n, Kp, pb);
  if (Kp > 6 * k) {
    long long pw = (long long)(Kp - 6 * k);
    launch_pdl(zero_pad, dim3((unsigned)(((long long)2 * n * pw + 255) / 256)), dim3(256), 0, s, pb, 2LL * n, 6 * k, Kp);
  }
  CUtensorMap ma, mb;
  if (!make_map(&ma, pa, m, Kp, tc::BM) || !make_map(&mb, pb, 2 * n, Kp, tc::BN)) return false;
  static bool attr = false;
  if (!attr) {
    *err = allow_max_smem(tc_gemm_kernel);
    if (*err != cudaSuccess) return false;
    attr = true;
  }
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  const int mt = (m + tc::BM - 1) / tc::BM, ntn = (2 * n + tc::BN - 1) / tc::BN;
  const int ntiles = mt * ntn;
  launch_pdl(tc_gemm_kernel, dim3(std::min(ntiles, nsm)), dim3(320), (size_t)tc::SMEM_BYTES, s, ma, mb, C, ldc, m, n,
             Kp / tc::BK, mt, ntiles);
  *err = cudaGetLastError();
  return *err == cudaSuccess;
}

// error word of the bounded waits (nonzero: a wait gave up)
int tc_gemm_error(bool reset) {
  int h = 0;
  cudaMemcpyFromSymbol(&h, g_tc_error, sizeof(int));
  if (reset) {
    int z = 0;
    cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int));
  }
  return h;
}

}  // namespace gbem
