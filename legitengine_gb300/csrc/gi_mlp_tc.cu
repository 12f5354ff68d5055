// gi_mlp_tc.cu -- fused reconstruction on the 5th-generation tensor cores: the
// 32 features of each pixel and the 32 -> 64 -> 64 -> 64 -> 3 network in one
// persistent kernel, with tcgen05.mma (BF16 operands from shared memory, FP32
// accumulators in tensor memory) and no intermediate buffer in HBM.
//
// One CTA per SM = 8 groups of 4 warps sharing one shared-memory copy of the
// weights and the SM's 512 tensor-memory columns; each group works on its own
// 128-pixel tile with its own A operand, staging buffer, mbarriers, named barrier
// and 64 columns, so the groups' feature gathers and MMA rounds overlap.  In a
// group, thread i owns pixel i of the tile, which is row i of every layer's A
// operand and lane i of the accumulator, so each warp reads back exactly its own
// 32 lanes.  Per tile:
//   features (registers) -> A [128 x 32] -> MMA with W1 (+ the bias MMA) ->
//   tcgen05.ld, ReLU, bf16 -> A [128 x 64] -> MMA with W2 -> ... -> MMA with W4
//   (N = 16, columns 3-15 unused) -> softmax blend of the candidate estimates,
//   x exposure scale -> out.
// A tile is 128 consecutive pixels, so its own depth moments, normals, albedo,
// few-ray light and direct light are five contiguous byte ranges: one thread of
// the group copies them into the group's staging buffer with bulk asynchronous
// copies (TMA, cp.async.bulk, completion counted in bytes on an mbarrier) for
// the NEXT tile while the current tile runs its MMA rounds; the neighbourhood
// and mip taps are read from global memory.  (Inputs not 16-byte aligned, and a
// last partial tile, read everything from global memory.)
// One thread of a group issues the MMAs of a layer, commits them to the group's
// mbarrier and waits on it, and waits for the staging copies (bounded: a wait
// that runs out records an error and the group stops; the CTA then waits for its
// copies in flight, frees its tensor memory and returns) while the group's other
// threads block on a hardware barrier.
//
// Operand layout: K-major without swizzle.  A core matrix is 8 rows x 16 bytes
// stored as 128 contiguous bytes; core matrices adjacent along K are 128 bytes
// apart (the descriptor's leading byte offset) and those adjacent along M (or N)
// are K*2*8 bytes apart (its stride byte offset).  One MMA consumes K = 16, so a
// layer of depth K is K/16 MMAs whose descriptors advance by 256 bytes.
#include <cuda_bf16.h>

#include <mutex>

#include "gi_features.cuh"
#include "gi_internal.h"
#include "gi_mlp.h"
#include "gi_mlp_layout.h"

namespace gi {
namespace {

using bf16 = __nv_bfloat16;

constexpr int kRows = 128;  // pixels per tile = MMA M = accumulator lanes
constexpr int kGroups = 8;  // tiles in flight per CTA (one CTA per SM)
constexpr int kTcThreads = 128 * kGroups;
constexpr uint32_t kTmemCols = 64 * kGroups;  // one 128 x 64 FP32 accumulator per group: all 512 columns

// Shared memory (bytes).  B operands are the weights as N x K (K-major).
constexpr int kB4Rows = 8;                        // W4 rows 0-7 (3 outputs, zero padding)
constexpr int tB1 = 0;                            // 64 x 32
constexpr int tB2 = tB1 + kHid * kIn * 2;         // 64 x 64
constexpr int tB3 = tB2 + kHid * kHid * 2;        // 64 x 64
constexpr int tB4 = tB3 + kHid * kHid * 2;        // 8 x 64; the MMA's rows 8-15 re-read rows 0-7
// Biases enter the accumulators through one extra MMA per layer: A = a constant
// "ones" operand, B = the bias operand.  Bias row n holds, at k = 2L and 2L + 1,
// the bf16 high and low parts of layer L's bias b_L[n] (b - hi rounded again), so
// the MMA adds hi + lo, b to about 2^-16 relative.  Layer L's ones operand has
// 1 at k = 2L, 2L + 1 in every row: one 8 x 8 core matrix read for all 16 row
// groups (stride byte offset 0), its k = 8-15 half a zero core matrix.
constexpr int tBB = tB4 + kB4Rows * kHid * 2;     // 64 rows x 8 k (16 bytes a row)
constexpr int tOnes = tBB + kHid * 16;            // 4 ones core matrices + 1 zero core matrix
constexpr int tA = tOnes + 5 * 128;               // per group 128 x 64 (layer 1 uses 128 x 32)
constexpr int kABytes = kRows * kHid * 2;
// Staging of a tile's own inputs: normal, albedo, few-ray light, direct light
// (16 bytes a pixel each) and depth moments (8).
constexpr int sNormal = 0, sAlbedo = 2048, sLight = 4096, sDirect = 6144, sMoments = 8192;
constexpr int kStageBytes = 9216;
constexpr int tStage = tA + kGroups * kABytes;
constexpr int tBar = tStage + kGroups * kStageBytes;  // per group: MMA mbarrier, staging mbarrier
constexpr int tFail = tBar + 16 * kGroups;            // one int per group
constexpr int tTmem = tFail + 4 * kGroups;
constexpr int kSmemTc = tTmem + 8;
static_assert(tStage % 128 == 0 && kStageBytes % 128 == 0, "bulk copy destinations");
static_assert(tBB % 128 == 0 && tOnes % 128 == 0 && tA % 128 == 0 && kABytes % 128 == 0 && tBar % 8 == 0,
              "alignment");

__device__ int g_tc_errors;  // waits that ran out (kept across launches)
constexpr long long kWaitCycles = 1ll << 31;  // ~1 s of SM clocks
// Bound of each tile group's first MMA-completion wait in a launch; kWaitCycles
// unless the test hook gi_debug_tensor_core_wait_limit shortened it (so that the
// wait runs out and the error path runs).  Every other wait keeps kWaitCycles.
__device__ long long g_tc_first_wait_cycles = kWaitCycles;

// Byte offset of element (r, k) of an R x K operand in the K-major core-matrix layout.
__device__ __forceinline__ int cm_off(int r, int k, int K) {
  return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (each stored >> 4), the fixed version bits 46-48 = 0b001, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// (bits 7-9 = 1) and B (bits 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Waits for the phase with the given parity to complete, for at most `limit` SM
// cycles (by default ~2^31, about a second); false if it did not.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit = kWaitCycles) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}

// One arrival that also expects `bytes` of asynchronous copies on the barrier.
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Bulk asynchronous copy global -> shared (TMA, no tensor map), completing
// `bytes` on the mbarrier; both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// 16 consecutive FP32 columns of this thread's accumulator lane; the load and
// its completion wait are one asm statement, so no use can be scheduled between.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive FP32 columns of this thread's accumulator lane (one load, one wait).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const bf16 x = __float2bfloat16_rn(a), y = __float2bfloat16_rn(b);
  return (uint32_t)__bfloat16_as_ushort(x) | ((uint32_t)__bfloat16_as_ushort(y) << 16);
}

// ReLU of two FP32 values rounded to bf16 and packed (a in the low half), one cvt.
__device__ __forceinline__ uint32_t pack_relu_bf16(float a, float b) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  return r;
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// Copies layer weights W [K x N] (row stride ldw, bf16, global) into the N x K
// K-major core-matrix layout at smem + off (rows n >= nvalid of W4 are the zero padding).
__device__ __forceinline__ void stage_b(unsigned char* smem, int off, const bf16* __restrict__ w, int K, int N,
                                        int ldw) {
  for (int i = threadIdx.x; i < K * N; i += kTcThreads) {
    const int k = i / N, n = i % N;
    *reinterpret_cast<bf16*>(smem + off + cm_off(n, k, K)) = w[k * ldw + n];
  }
}

// Barrier of one group's 128 threads (named barrier 1 + group).
__device__ __forceinline__ void group_sync(int group) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + group), "r"(kRows) : "memory");
}

// Makes this group's A operand visible to the tensor cores, issues the layer's
// bias MMA and its K/16 MMAs from the group's first thread, which alone waits for their
// completion (the other 127 threads block on the group's hardware barrier instead
// of spinning); the fence pair around that barrier orders the completion before
// every thread's accumulator reads.  Returns false (on every thread of the group)
// if the wait ran out.
// The B operand's row-group stride is K * 16 bytes, or 0 when its N = 16 rows
// re-read the first 8 (the output layer).
// `first` runs on the issuing thread after the barrier, before the MMAs.
template <int K, int N, int L, typename First>
__device__ __forceinline__ bool run_layer(uint32_t sbase, int a_off, int b_off, uint32_t tmem, uint32_t bar,
                                          uint32_t& phase, int group, volatile int* fail, First first,
                                          long long limit = kWaitCycles) {
  fence_async_smem();
  fence_before();
  group_sync(group);
  fence_after();
  if ((threadIdx.x & (kRows - 1)) == 0) {
    first();
    constexpr uint32_t idesc = idesc_bf16(kRows, N);
    constexpr uint32_t b_sbo = (N == kOutPad) ? 0u : (uint32_t)(K * 16);
    mma_bf16(tmem, smem_desc(sbase + tOnes + 128 * L, 512 - 128 * L, 0), smem_desc(sbase + tBB, 0, 128), idesc, 0u);
#pragma unroll
    for (int j = 0; j < K / 16; j++) {
      const uint64_t ad = smem_desc(sbase + a_off + j * 256, 128, K * 16);
      const uint64_t bd = smem_desc(sbase + b_off + j * 256, 128, b_sbo);
      mma_bf16(tmem, ad, bd, idesc, 1u);
    }
    mma_commit(bar);
    if (!mbar_wait(bar, phase, limit)) *fail = 1;
    fence_before();
  }
  phase ^= 1u;
  group_sync(group);
  const bool failed = *fail != 0;
  fence_after();
  return !failed;
}

// Hidden-layer epilogue: accumulator lane (bias included) -> ReLU -> bf16 row
// of the next A operand (K = 64).
__device__ __forceinline__ void hidden_epilogue(uint32_t a_base, uint32_t taddr) {
  const int m = threadIdx.x & (kRows - 1);
#pragma unroll
  for (int c = 0; c < kHid; c += 32) {
    float v[32];
    tmem_ld32(taddr + c, v);
#pragma unroll
    for (int h = 0; h < 4; h++) {
      const int k = c + 8 * h;
      st_shared_v4(a_base + cm_off(m, k, kHid), pack_relu_bf16(v[8 * h + 0], v[8 * h + 1]),
                   pack_relu_bf16(v[8 * h + 2], v[8 * h + 3]), pack_relu_bf16(v[8 * h + 4], v[8 * h + 5]),
                   pack_relu_bf16(v[8 * h + 6], v[8 * h + 7]));
    }
  }
}

// Issues the staging copies of tile t (a full tile) into the group's buffer.
__device__ __forceinline__ void stage_tile(const FeatureArgs& a, int t, uint32_t buf, uint32_t bar) {
  const size_t p0 = (size_t)t * kRows;
  fence_async_smem();  // the group's reads of the previous tile's staging come first
  mbar_expect_tx(bar, kStageBytes);
  bulk_g2s(buf + sNormal, a.normal + 4 * p0, 16 * kRows, bar);
  bulk_g2s(buf + sAlbedo, a.albedo + 4 * p0, 16 * kRows, bar);
  bulk_g2s(buf + sLight, a.indirect[0] + 4 * p0, 16 * kRows, bar);
  bulk_g2s(buf + sDirect, a.direct + 4 * p0, 16 * kRows, bar);
  bulk_g2s(buf + sMoments, a.moments + 2 * p0, 8 * kRows, bar);
}

// ROWS: the network on given feature rows (a.rows, a.row_scale; a.width = rows,
// a.height = 1) instead of the fused feature builder -- the same MMA rounds,
// epilogues and head.
template <bool ROWS>
__global__ void __launch_bounds__(kTcThreads, 1) mlp_reconstruct_kernel(const __grid_constant__ FeatureArgs a,
                                                                     const bf16* __restrict__ wb,
                                                                     const float* __restrict__ params,
                                                                     float* __restrict__ out, int staged) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int group = tid / kRows, gtid = tid % kRows;
  const uint32_t sbase = smem_u32(smem);
  const uint32_t bar = sbase + tBar + 16 * group;  // MMA completion
  const uint32_t sbar = bar + 8;                   // staging copies
  const uint32_t stage = sbase + tStage + group * kStageBytes;
  const unsigned char* stage_p = smem + tStage + group * kStageBytes;
  const int a_off = tA + group * kABytes;
  volatile int* fail = reinterpret_cast<volatile int*>(smem + tFail) + group;

  stage_b(smem, tB1, wb + qW1, kIn, kHid, kHid);
  stage_b(smem, tB2, wb + qW2, kHid, kHid, kHid);
  stage_b(smem, tB3, wb + qW3, kHid, kHid, kHid);
  stage_b(smem, tB4, wb + qW4, kHid, kB4Rows, kOutPad);
  // Bias operand: row n, k = 2L / 2L + 1 = high / low bf16 part of b_L[n].
  for (int i = tid; i < kHid * 8; i += kTcThreads) {
    const int n = i >> 3, k = i & 7, L = k >> 1;
    float b = 0.0f;
    if (L == 0) b = params[ob1 + n];
    else if (L == 1) b = params[ob2 + n];
    else if (L == 2) b = params[ob3 + n];
    else if (n < kOut) b = params[ob4 + n];
    const bf16 hi = __float2bfloat16_rn(b);
    const bf16 v = (k & 1) ? __float2bfloat16_rn(b - __bfloat162float(hi)) : hi;
    *reinterpret_cast<bf16*>(smem + tBB + n * 16 + k * 2) = v;
  }
  // Ones operands: core matrix L (8 rows x 8 k) is 1 at k = 2L, 2L + 1; core 4 is zero.
  for (int i = tid; i < 5 * 64; i += kTcThreads) {
    const int L = i >> 6, k = i & 7;
    *reinterpret_cast<bf16*>(smem + tOnes + 2 * i) = __float2bfloat16_rn((L < 4 && (k >> 1) == L) ? 1.0f : 0.0f);
  }
  if (gtid == 0) {
    mbar_init(bar, 1);
    mbar_init(sbar, 1);
    *fail = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + tTmem),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();  // the staged operands, for the tensor cores
  fence_before();
  __syncthreads();
  fence_after();
  // This group's 64 accumulator columns; this warp's 32 lanes of them.
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + tTmem) + (uint32_t)(64 * group);
  const uint32_t lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16);

  const int W = a.width, n = a.width * a.height;
  const int tiles = (n + kRows - 1) / kRows;
  const int full_tiles = n / kRows;
  const int stride = gridDim.x * kGroups;
  uint32_t phase = 0, sphase = 0;
  bool failed = false;
  int t = blockIdx.x * kGroups + group;
  const int first_tile = t;
  bool pending = staged && t < full_tiles;  // a staging copy of tile t in flight
  if (pending && gtid == 0) stage_tile(a, t, stage, sbar);
  for (; t < tiles && !failed; t += stride) {
    const int p = t * kRows + gtid;
    float f[kIn];
    float scale = 1.0f;
    if (ROWS) {  // the row's bf16 features (exact in float) and its scale
      if (p < n) {
        const uint4* src = reinterpret_cast<const uint4*>(a.rows + (size_t)p * kIn);
#pragma unroll
        for (int c = 0; c < kIn / 8; c++) {
          const uint4 q = __ldg(src + c);
          const uint32_t w4[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
          for (int h = 0; h < 4; h++) {
            f[8 * c + 2 * h] = __uint_as_float(w4[h] << 16);
            f[8 * c + 2 * h + 1] = __uint_as_float(w4[h] & 0xFFFF0000u);
          }
        }
        if (a.row_scale) scale = __ldg(a.row_scale + p);
      } else {
#pragma unroll
        for (int i = 0; i < kIn; i++) f[i] = 0.0f;
      }
    } else if (pending) {
      if (gtid == 0 && !mbar_wait(sbar, sphase)) *fail = 1;
      group_sync(group);
      if (*fail) { failed = true; break; }  // the copy stays pending: waited for again before exit
      sphase ^= 1u;
      pending = false;
      const float depth = reinterpret_cast<const float*>(stage_p + sMoments)[2 * gtid];
      const float4 n4 = reinterpret_cast<const float4*>(stage_p + sNormal)[gtid];
      const float4 al = reinterpret_cast<const float4*>(stage_p + sAlbedo)[gtid];
      const float4 li = reinterpret_cast<const float4*>(stage_p + sLight)[gtid];
      const float4 dl = reinterpret_cast<const float4*>(stage_p + sDirect)[gtid];
      pixel_features_from(a, p % W, p / W, depth, n4, al, li, dl, f, scale);
    } else if (p < n) {
      pixel_features(a, p % W, p / W, f, scale);
    } else {
#pragma unroll
      for (int i = 0; i < kIn; i++) f[i] = 0.0f;
    }
    // The staging buffer takes the group's next tile once every thread has its
    // features: issued after the first layer's barrier.
    const bool prefetch = staged && t + stride < full_tiles;
    pending = prefetch;
#pragma unroll
    for (int c = 0; c < kIn; c += 8)
      st_shared_v4(sbase + a_off + cm_off(gtid, c, kIn), pack_bf16(f[c], f[c + 1]), pack_bf16(f[c + 2], f[c + 3]),
                   pack_bf16(f[c + 4], f[c + 5]), pack_bf16(f[c + 6], f[c + 7]));
    // The head blends candidate estimates as the network saw them (bf16).
    float cand[3][3];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      cand[0][ch] = __bfloat162float(__float2bfloat16_rn(f[kCand0 + ch]));
      cand[1][ch] = __bfloat162float(__float2bfloat16_rn(f[kCand1 + ch]));
      cand[2][ch] = __bfloat162float(__float2bfloat16_rn(f[kCand2 + ch]));
    }

    const int tn = t + stride;
    auto issue_next = [&] {
      if (prefetch) stage_tile(a, tn, stage, sbar);
    };
    auto nothing = [] {};
    const long long first_limit = t == first_tile ? g_tc_first_wait_cycles : kWaitCycles;
    if (!run_layer<kIn, kHid, 0>(sbase, a_off, tB1, tmem, bar, phase, group, fail, issue_next, first_limit)) {
      failed = true;
      break;
    }
    hidden_epilogue(sbase + a_off, lane_addr);
    if (!run_layer<kHid, kHid, 1>(sbase, a_off, tB2, tmem, bar, phase, group, fail, nothing)) { failed = true; break; }
    hidden_epilogue(sbase + a_off, lane_addr);
    if (!run_layer<kHid, kHid, 2>(sbase, a_off, tB3, tmem, bar, phase, group, fail, nothing)) { failed = true; break; }
    hidden_epilogue(sbase + a_off, lane_addr);
    if (!run_layer<kHid, kOutPad, 3>(sbase, a_off, tB4, tmem, bar, phase, group, fail, nothing)) {
      failed = true;
      break;
    }
    float v[16];
    tmem_ld16(lane_addr, v);
    if (p < n) {
      const float lo[3] = {v[0], v[1], v[2]};
      float w[3], y[3];
      head_forward(lo, cand, w, y);
      reinterpret_cast<float4*>(out)[p] = make_float4(y[0] * scale, y[1] * scale, y[2] * scale, 1.0f);
    }
  }
  if (failed && gtid == 0) {
    atomicAdd(&g_tc_errors, 1);
    (void)mbar_wait(bar, phase ^ 1u);  // the group's MMAs in flight, bounded
  }
  if (pending && gtid == 0) (void)mbar_wait(sbar, sphase);  // a staging copy in flight, bounded
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem - (uint32_t)(64 * group)),
                 "r"(kTmemCols)
                 : "memory");
}

// ---- Training on the tensor cores -----------------------------------------
//
// mlp_train_tc_kernel: forward with saved activations, the head's loss gradient,
// backward through every layer and the weight gradients, for 128-pixel tiles
// (persistent: one CTA of 128 threads per SM walks the batch's tiles).  Thread i
// owns pixel i of a tile: row i of every layer's A operand and lane i of the
// accumulators.  Products of a tile (A = M x K, B = N x K, both K-major without
// swizzle, D in tensor memory, M = 128):
//   forward   Z = A_l W_l             A = X / H1 / H2 / H3 (pixels x features)
//   backward  dH = dZ_l W_l^T         A = dZ (pixels x outputs), B = W_l as (in x out)
//   gradient  dW_l += H_{l-1}^T dZ_l  A = H^T (features x pixels), B = dZ^T
//                                     (outputs x pixels): the pixels are the
//                                     reduction, and dW accumulates over every
//                                     tile of the CTA in tensor memory (M = 128:
//                                     rows past the layer's inputs read the
//                                     next buffer and are never read back).
// Epilogues (one thread per pixel, its own accumulator lane): bias and ReLU to
// bf16 (forward; the transposed copy H^T written beside the row), the head's
// loss gradient (layer 4), the ReLU mask of the backward (dZ = dH where H > 0).
// Bias gradients are the column sums of the bf16 dZ (shared memory).  At the end
// each CTA adds its gradient sums to `grads` (atomic FP32 additions) and its loss.
// Arithmetic: bf16 operands (inputs, weights, hidden activations, the logits'
// gradient and the masked hidden gradients), FP32 accumulation, FP32 bias and
// head; the sums run in the tensor cores' order.
constexpr int kTrThreads = 128;
constexpr int uF1 = 0;                            // W1 as 64 x 32 (out x in)
constexpr int uF2 = uF1 + kHid * kIn * 2;          // W2 as 64 x 64
constexpr int uF3 = uF2 + kHid * kHid * 2;
constexpr int uF4 = uF3 + kHid * kHid * 2;         // W4 as 16 x 64 (rows 3-15 zero)
constexpr int uB2 = uF4 + kOutPad * kHid * 2;      // W2 as 64 x 64 (in x out)
constexpr int uB3 = uB2 + kHid * kHid * 2;
constexpr int uB4 = uB3 + kHid * kHid * 2;         // W4 as 64 x 16 (in x out, outputs 3-15 zero)
constexpr int uX = uB4 + kHid * kOutPad * 2;       // 128 x 32
constexpr int uH1 = uX + kRows * kIn * 2;          // 128 x 64 each
constexpr int uH2 = uH1 + kRows * kHid * 2;
constexpr int uH3 = uH2 + kRows * kHid * 2;
constexpr int uDY = uH3 + kRows * kHid * 2;        // 128 x 16
constexpr int uDZ = uDY + kRows * kOutPad * 2;     // 128 x 64
constexpr int uXt = uDZ + kRows * kHid * 2;        // 32 x 128 (features x pixels)
constexpr int uH1t = uXt + kIn * kRows * 2;        // 64 x 128 each
constexpr int uH2t = uH1t + kHid * kRows * 2;
constexpr int uH3t = uH2t + kHid * kRows * 2;
constexpr int uDZt = uH3t + kHid * kRows * 2;      // 64 x 128 (outputs x pixels)
constexpr int uDYt = uDZt + kHid * kRows * 2;      // 16 x 128
constexpr int uBar = uDYt + kOutPad * kRows * 2;
constexpr int uFail = uBar + 8;
constexpr int uTmem = uFail + 4;
constexpr int kSmemTrainTc = uTmem + 4;
// A 128-row gradient operand reads 128 rows of 256 bytes from its start: the
// buffers after Xt (24 KB) and after each H^T (16 KB) stay inside the allocation.
static_assert(uXt + kRows * kRows * 2 <= kSmemTrainTc && uH3t + kRows * kRows * 2 <= kSmemTrainTc,
              "gradient operand reads stay in shared memory");
static_assert(uX % 128 == 0 && uDY % 128 == 0 && uXt % 128 == 0 && uDYt % 128 == 0 && uBar % 8 == 0, "alignment");
// Tensor-memory columns: the layer accumulator and the four weight-gradient sums.
constexpr uint32_t cZ = 0, cW1 = 64, cW2 = 128, cW3 = 192, cW4 = 256, kTrTmemCols = 512;

// Element (r, k) of an R x K K-major operand, as bf16 at smem + base.
__device__ __forceinline__ void st_bf16(unsigned char* smem, int base, int r, int k, int K, bf16 v) {
  *reinterpret_cast<bf16*>(smem + base + cm_off(r, k, K)) = v;
}

// Row `m` of a 128 x K operand from 8-value packs (v4 stores).
template <int K>
__device__ __forceinline__ void st_row(uint32_t sbase, int base, int m, const uint32_t (&packs)[K / 2]) {
#pragma unroll
  for (int c = 0; c < K; c += 8)
    st_shared_v4(sbase + base + cm_off(m, c, K), packs[c / 2], packs[c / 2 + 1], packs[c / 2 + 2], packs[c / 2 + 3]);
}

// Column `m` of the transposed K x 128 operand (one bf16 per feature).
template <int K>
__device__ __forceinline__ void st_col(unsigned char* smem, int base, int m, const uint32_t (&packs)[K / 2]) {
#pragma unroll
  for (int k = 0; k < K; k++) {
    const uint32_t w = packs[k / 2];
    const unsigned short h = (k & 1) ? (unsigned short)(w >> 16) : (unsigned short)(w & 0xFFFFu);
    *reinterpret_cast<unsigned short*>(smem + base + cm_off(k, m, kRows)) = h;
  }
}

// K/16 MMAs of A (M = 128 x K) and B (N x K) into D; `first` clears D.
template <int K, int N>
__device__ __forceinline__ void mma_chain(uint32_t d, uint32_t a, uint32_t b, bool first) {
  constexpr uint32_t idesc = idesc_bf16(kRows, N);
#pragma unroll
  for (int j = 0; j < K / 16; j++)
    mma_bf16(d, smem_desc(a + j * 256, 128, K * 16), smem_desc(b + j * 256, 128, K * 16), idesc,
             (first && j == 0) ? 0u : 1u);
}

__global__ void __launch_bounds__(kTrThreads, 1) mlp_train_tc_kernel(const bf16* __restrict__ feats,
                                                                   const float* __restrict__ targets,
                                                                   const float* __restrict__ scale, int n,
                                                                   const bf16* __restrict__ wb,
                                                                   const float* __restrict__ params,
                                                                   float* __restrict__ grads,
                                                                   float* __restrict__ loss, int loss_kind) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t sbase = smem_u32(smem);
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t bar = sbase + uBar;
  volatile int* fail = reinterpret_cast<volatile int*>(smem + uFail);

  // Weights: forward B (out x in) and backward B (in x out), K-major.
  for (int i = tid; i < kHid * kIn; i += kTrThreads) {  // W1 [32 x 64]
    const int k = i / kHid, o = i % kHid;
    st_bf16(smem, uF1, o, k, kIn, wb[qW1 + i]);
  }
  for (int i = tid; i < kHid * kHid; i += kTrThreads) {
    const int k = i / kHid, o = i % kHid;
    st_bf16(smem, uF2, o, k, kHid, wb[qW2 + i]);
    st_bf16(smem, uF3, o, k, kHid, wb[qW3 + i]);
    st_bf16(smem, uB2, k, o, kHid, wb[qW2 + i]);
    st_bf16(smem, uB3, k, o, kHid, wb[qW3 + i]);
  }
  for (int i = tid; i < kHid * kOutPad; i += kTrThreads) {  // W4 [64 x 16]
    const int k = i / kOutPad, o = i % kOutPad;
    st_bf16(smem, uF4, o, k, kHid, wb[qW4 + i]);
    st_bf16(smem, uB4, k, o, kOutPad, wb[qW4 + i]);
  }
  for (int i = tid; i < kOutPad * kRows; i += kTrThreads)  // dY^T: outputs 3-15 stay zero
    *reinterpret_cast<bf16*>(smem + uDYt + 2 * i) = __float2bfloat16_rn(0.0f);
  if (tid == 0) {
    mbar_init(bar, 1);
    *fail = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + uTmem),
                 "r"(kTrTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(smem + uTmem);
  const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 accumulator lanes
  uint32_t phase = 0;
  bool failed = false, first = true;
  float lsum = 0.0f, gb1 = 0.0f, gb2 = 0.0f, gb3 = 0.0f, gb4 = 0.0f;
  const float b40 = params[ob4 + 0], b41 = params[ob4 + 1], b42 = params[ob4 + 2];

  // Shared-memory writes -> the tensor cores -> `issue` on thread 0 -> commit, wait.
  auto mma_round = [&](auto issue) {
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    if (tid == 0) {
      issue();
      mma_commit(bar);
      if (!mbar_wait(bar, phase)) *fail = 1;
      fence_before();
    }
    phase ^= 1u;
    __syncthreads();
    fence_after();
    return *fail == 0;
  };
  // Layer accumulator -> + bias -> ReLU -> bf16 row and column of the next operand.
  auto forward_epilogue = [&](int row_buf, int col_buf, const float* __restrict__ bias) {
    uint32_t packs[kHid / 2];
#pragma unroll
    for (int c = 0; c < kHid; c += 32) {
      float v[32];
      tmem_ld32(lane + cZ + c, v);
#pragma unroll
      for (int h = 0; h < 32; h += 2)
        packs[(c + h) / 2] = pack_relu_bf16(v[h] + __ldg(bias + c + h), v[h + 1] + __ldg(bias + c + h + 1));
    }
    st_row<kHid>(sbase, row_buf, tid, packs);
    st_col<kHid>(smem, col_buf, tid, packs);
  };
  // dH (accumulator) masked by the ReLU of the layer's output (bf16 row in smem) -> dZ.
  auto backward_epilogue = [&](int h_buf) {
    uint32_t packs[kHid / 2];
#pragma unroll
    for (int c = 0; c < kHid; c += 32) {
      float v[32];
      tmem_ld32(lane + cZ + c, v);
#pragma unroll
      for (int h = 0; h < 32; h += 2) {
        const uint32_t hp =
            *reinterpret_cast<const uint32_t*>(smem + h_buf + cm_off(tid, c + h, kHid));  // H[tid][c+h], [c+h+1]
        const float g0 = (hp & 0xFFFFu) && !(hp & 0x8000u) ? v[h] : 0.0f;      // bf16 > 0
        const float g1 = (hp >> 16) && !(hp & 0x80000000u) ? v[h + 1] : 0.0f;
        packs[(c + h) / 2] = pack_bf16(g0, g1);
      }
    }
    st_row<kHid>(sbase, uDZ, tid, packs);
    st_col<kHid>(smem, uDZt, tid, packs);
  };
  // Column sum of the bf16 dZ rows (threads 0..cols-1), after the rows are written.
  auto column_sum = [&](int buf, int K, int cols) {
    float sum = 0.0f;
    if (tid < cols)
      for (int r = 0; r < kRows; r++) sum += __bfloat162float(*reinterpret_cast<const bf16*>(smem + buf + cm_off(r, tid, K)));
    return sum;
  };

  const int tiles = (n + kRows - 1) / kRows;
  for (int t = blockIdx.x; t < tiles && !failed; t += gridDim.x) {
    const int p = t * kRows + tid;
    const bool valid = p < n;
    // Features: row and column of X; targets divided by the exposure scale.
    uint32_t xp[kIn / 2];
    {
      const uint4* src = reinterpret_cast<const uint4*>(feats + (size_t)p * kIn);
#pragma unroll
      for (int c = 0; c < kIn / 8; c++) {
        const uint4 q = valid ? __ldg(src + c) : make_uint4(0u, 0u, 0u, 0u);
        xp[4 * c] = q.x;
        xp[4 * c + 1] = q.y;
        xp[4 * c + 2] = q.z;
        xp[4 * c + 3] = q.w;
      }
    }
    st_row<kIn>(sbase, uX, tid, xp);
    st_col<kIn>(smem, uXt, tid, xp);
    float T[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (valid) {
      const float sc = scale ? __ldg(scale + p) : 1.0f;
#pragma unroll
      for (int c = 0; c < 3; c++) T[c] = scale ? __ldg(targets + (size_t)p * 4 + c) / sc : __ldg(targets + (size_t)p * 4 + c);
      T[3] = __ldg(targets + (size_t)p * 4 + 3);
    }
    auto xval = [&](int k) {
      const uint32_t w = xp[k / 2];
      return __uint_as_float(((k & 1) ? (w >> 16) : (w & 0xFFFFu)) << 16);
    };

    if (!mma_round([&] { mma_chain<kIn, kHid>(tmem + cZ, sbase + uX, sbase + uF1, true); })) break;
    forward_epilogue(uH1, uH1t, params + ob1);
    if (!mma_round([&] { mma_chain<kHid, kHid>(tmem + cZ, sbase + uH1, sbase + uF2, true); })) break;
    forward_epilogue(uH2, uH2t, params + ob2);
    if (!mma_round([&] { mma_chain<kHid, kHid>(tmem + cZ, sbase + uH2, sbase + uF3, true); })) break;
    forward_epilogue(uH3, uH3t, params + ob3);
    if (!mma_round([&] { mma_chain<kHid, kOutPad>(tmem + cZ, sbase + uH3, sbase + uF4, true); })) break;
    // Head: the loss gradient at the logits -> dY (row and column).
    {
      float z[16];
      tmem_ld16(lane + cZ, z);
      const float lo[3] = {z[0] + b40, z[1] + b41, z[2] + b42};
      float c[3][3], d[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        c[0][ch] = xval(kCand0 + ch);
        c[1][ch] = xval(kCand1 + ch);
        c[2][ch] = xval(kCand2 + ch);
      }
      const float l = head_loss_grad_logits(lo, c, T, d, loss_kind);
      if (valid) lsum += l;
      else d[0] = d[1] = d[2] = 0.0f;
      uint32_t dy[kOutPad / 2] = {pack_bf16(d[0], d[1]), pack_bf16(d[2], 0.0f), 0u, 0u, 0u, 0u, 0u, 0u};
      st_row<kOutPad>(sbase, uDY, tid, dy);
#pragma unroll
      for (int o = 0; o < 3; o++)
        st_bf16(smem, uDYt, o, tid, kRows, __float2bfloat16_rn(d[o]));
    }
    // Layer 4: dW4 += H3^T dY, dH3 = dY W4^T.
    if (!mma_round([&] {
          mma_chain<kRows, kOutPad>(tmem + cW4, sbase + uH3t, sbase + uDYt, first);
          mma_chain<kOutPad, kHid>(tmem + cZ, sbase + uDY, sbase + uB4, true);
        }))
      break;
    gb4 += column_sum(uDY, kOutPad, kOut);
    backward_epilogue(uH3);
    __syncthreads();
    gb3 += column_sum(uDZ, kHid, kHid);
    // Layer 3: dW3 += H2^T dZ3, dH2 = dZ3 W3^T.
    if (!mma_round([&] {
          mma_chain<kRows, kHid>(tmem + cW3, sbase + uH2t, sbase + uDZt, first);
          mma_chain<kHid, kHid>(tmem + cZ, sbase + uDZ, sbase + uB3, true);
        }))
      break;
    backward_epilogue(uH2);
    __syncthreads();
    gb2 += column_sum(uDZ, kHid, kHid);
    // Layer 2: dW2 += H1^T dZ2, dH1 = dZ2 W2^T.
    if (!mma_round([&] {
          mma_chain<kRows, kHid>(tmem + cW2, sbase + uH1t, sbase + uDZt, first);
          mma_chain<kHid, kHid>(tmem + cZ, sbase + uDZ, sbase + uB2, true);
        }))
      break;
    backward_epilogue(uH1);
    __syncthreads();
    gb1 += column_sum(uDZ, kHid, kHid);
    // Layer 1: dW1 += X^T dZ1.
    if (!mma_round([&] { mma_chain<kRows, kHid>(tmem + cW1, sbase + uXt, sbase + uDZt, first); })) break;
    first = false;
  }
  failed = *fail != 0;
  if (failed && tid == 0) {
    atomicAdd(&g_tc_errors, 1);
    (void)mbar_wait(bar, phase ^ 1u);  // the MMAs in flight, bounded
  }
  if (!failed && !first) {
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((tid & 31) == 0) atomicAdd(loss, lsum);
    if (tid < kHid) {
      atomicAdd(grads + ob1 + tid, gb1);
      atomicAdd(grads + ob2 + tid, gb2);
      atomicAdd(grads + ob3 + tid, gb3);
    }
    if (tid < kOut) atomicAdd(grads + ob4 + tid, gb4);
    // Weight-gradient rows: lane r of the accumulators = input feature r.
    if (warp < 2) {
      auto add_rows = [&](uint32_t col, int rows, int N, float* g) {
#pragma unroll
        for (int c = 0; c < kHid; c += 32) {
          if (c >= N) break;
          float v[32];
          tmem_ld32(lane + col + c, v);
          if (tid < rows)
            for (int j = 0; j < 32 && c + j < N; j++) atomicAdd(g + tid * N + c + j, v[j]);
        }
      };
      add_rows(cW1, kIn, kHid, grads + oW1);
      add_rows(cW2, kHid, kHid, grads + oW2);
      add_rows(cW3, kHid, kHid, grads + oW3);
      {
        float v[16];
        tmem_ld16(lane + cW4, v);
        if (tid < kHid)
          for (int j = 0; j < kOut; j++) atomicAdd(grads + oW4 + tid * kOut + j, v[j]);
      }
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTrTmemCols) : "memory");
}

std::mutex g_tc_mutex;
int g_tc_grid[64] = {0};  // persistent grid per device (0 = not set up)

}  // namespace

// The reconstruction kernels' shared-memory attributes, set once per device, and
// their persistent grid: one CTA per SM (each allocates all 512 tensor-memory columns).
static int reconstruct_grid_cap(int* cap) {
  int dev = 0;
  int e = check_cuda(cudaGetDevice(&dev), "reconstruct: device");
  if (e) return e;
  std::lock_guard<std::mutex> lock(g_tc_mutex);
  if (dev >= 64) return fail(GI_ERR_UNSUPPORTED, "reconstruct: device index");
  if (!g_tc_grid[dev]) {
    int sms = 0, optin = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (optin < kSmemTc) return fail(GI_ERR_UNSUPPORTED, "reconstruct: not enough shared memory per block");
    for (auto kernel : {mlp_reconstruct_kernel<false>, mlp_reconstruct_kernel<true>}) {
      e = check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTc),
                     "reconstruct: smem attribute");
      if (e) return e;
      e = check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
                     "reconstruct: carveout");
      if (e) return e;
    }
    g_tc_grid[dev] = sms;
  }
  *cap = g_tc_grid[dev];
  return GI_OK;
}

int launch_reconstruct(const FeatureArgs& a, const __nv_bfloat16* wb, const float* params, float* out,
                       cudaStream_t stream) {
  int grid_cap = 0;
  int e = reconstruct_grid_cap(&grid_cap);
  if (e) return e;
  const int n = a.width * a.height;
  const int tiles = (n + kRows - 1) / kRows;
  const int ctas = (tiles + kGroups - 1) / kGroups;
  const int grid = ctas < grid_cap ? ctas : grid_cap;
  if (grid <= 0) return GI_OK;
  // The staging copies need 16-byte aligned sources.
  const int staged = aligned16(a.normal) && aligned16(a.albedo) && aligned16(a.indirect[0]) && aligned16(a.direct) &&
                     aligned16(a.moments);
  mlp_reconstruct_kernel<false><<<grid, kTcThreads, kSmemTc, stream>>>(a, wb, params, out, staged);
  GI_CHECK_LAUNCH("mlp_reconstruct_kernel");
  count_launches(1);
  return GI_OK;
}

int launch_forward_tc(const __nv_bfloat16* rows, const float* scale, int n, const __nv_bfloat16* wb,
                      const float* params, float* out, cudaStream_t stream) {
  if (n <= 0) return GI_OK;
  int grid_cap = 0;
  int e = reconstruct_grid_cap(&grid_cap);
  if (e) return e;
  FeatureArgs a{};
  a.width = n;
  a.height = 1;
  a.pattern = 1;
  a.rows = rows;
  a.row_scale = scale;
  const int tiles = (n + kRows - 1) / kRows;
  const int ctas = (tiles + kGroups - 1) / kGroups;
  const int grid = ctas < grid_cap ? ctas : grid_cap;
  mlp_reconstruct_kernel<true><<<grid, kTcThreads, kSmemTc, stream>>>(a, wb, params, out, 0);
  GI_CHECK_LAUNCH("mlp_reconstruct_kernel (rows)");
  count_launches(1);
  return GI_OK;
}

int launch_train_tc(const __nv_bfloat16* feats, const float* targets, const float* scale, int n,
                    const __nv_bfloat16* wb, const float* params, float* grads, float* loss, int loss_kind,
                    cudaStream_t stream) {
  int dev = 0;
  int e = check_cuda(cudaGetDevice(&dev), "train: device");
  if (e) return e;
  static bool attr_set[64] = {};
  int sms = 0;
  {
    std::lock_guard<std::mutex> lock(g_tc_mutex);
    if (dev >= 64) return fail(GI_ERR_UNSUPPORTED, "train: device index");
    if (!attr_set[dev]) {
      int optin = 0;
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      if (optin < kSmemTrainTc) return fail(GI_ERR_UNSUPPORTED, "train: not enough shared memory per block");
      e = check_cuda(cudaFuncSetAttribute(mlp_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          kSmemTrainTc),
                     "train: smem attribute");
      if (e) return e;
      attr_set[dev] = true;
    }
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const int tiles = (n + kRows - 1) / kRows;
  const int grid = tiles < sms ? tiles : sms;  // one CTA per SM: all 512 tensor-memory columns
  if (grid <= 0) return GI_OK;
  mlp_train_tc_kernel<<<grid, kTrThreads, kSmemTrainTc, stream>>>(feats, targets, scale, n, wb, params, grads,
                                                                   loss, loss_kind);
  GI_CHECK_LAUNCH("mlp_train_tc_kernel");
  count_launches(1);
  return GI_OK;
}

int reconstruct_wait_limit(long long cycles) {
  const long long v = cycles > 0 ? cycles : kWaitCycles;
  return check_cuda(cudaMemcpyToSymbol(g_tc_first_wait_cycles, &v, sizeof(v)), "reconstruct: wait limit");
}

int reconstruct_errors(int* count) {
  return check_cuda(cudaMemcpyFromSymbol(count, g_tc_errors, sizeof(int)), "reconstruct: error count");
}

}  // namespace gi
