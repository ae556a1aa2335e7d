// Fifth-generation tensor core (tcgen05) primitives for sm_103a, as inline PTX:
// tensor-memory allocation, the single-thread MMA issue of kind::tf32 with FP32
// accumulators in tensor memory, its completion through an mbarrier, and the
// tensor-memory loads of the epilogue.  Operands are staged by the threads in
// shared memory in the canonical K-major layout without swizzling: core
// matrices of 8 rows × 16 bytes (8 × 4 FP32), each 128 contiguous bytes, the
// core matrices along K `lbo` bytes apart and those along M (or N) `sbo` bytes
// apart.
#pragma once
#include <cstdint>

namespace mgpu {
namespace tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) of a K-major operand tile with kcols columns of K
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int kcols) {
  return uint32_t(((r >> 3) * (kcols >> 2) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

// shared memory matrix descriptor: start address, leading (K) and stride (M/N)
// byte offsets, descriptor version 1, no swizzling
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = uint64_t((saddr >> 4) & 0x3FFFu);
  d |= uint64_t((lbo >> 4) & 0x3FFFu) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFFu) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

// instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, M × N
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// TF32 part of x (round to nearest, ties away) and the remainder, itself
// rounded to TF32 (the tensor core would otherwise truncate it, a one-sided
// error that accumulates over the updates of a front)
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(x - hi));
  lo = __uint_as_float(l);
}

// ---- tensor memory (warp-wide: all 32 lanes of one warp)
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes to shared memory made visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- MMA (one thread)
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive on the mbarrier when every MMA this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// ---- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// bounded wait for the given phase: false when it did not complete in time
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, int64_t max_polls = int64_t(1) << 24) {
  for (int64_t i = 0; i < max_polls; ++i) {
    if (mbar_try_wait(bar, phase)) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

// ---- tensor memory loads: thread l of warp w gets lane 32 (w % 4) + l, 16 columns from `taddr`
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  // the load and its wait in one statement: the registers are defined only after the wait
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// ---- C tile −= A · B on the tensor cores, FP32 accuracy from three TF32 products
// C[i0 .. i0+128) × [j0 .. j0+128) −= A[·, 0..kb) · B[0..kb, ·] for kb ≤ 64, with
// A(i, k) = A[i + k·lda], B(k, j) = B[k + j·ldb], C(i, j) = C[i + j·ldc], rows
// below mrows and columns below ncols.  Each operand is split as x = hi + lo
// (hi its TF32 rounding) and the accumulator takes Aₕ·Bₕ + Aₕ·Bₗ + Aₗ·Bₕ.
// 128 threads; smem: 64 KB (the four split operand tiles of one K half of 32),
// 128-byte aligned; bar, tslot: shared.  Warp 0 holds 128 tensor-memory
// columns for the 128 × 128 FP32 accumulator (row i in lane i) and frees them
// before returning.  Returns false when the MMAs did not complete within the
// bounded wait (then C is left unchanged).
constexpr int kTcTile = 128;
constexpr int kTcThreads = 128;
constexpr size_t kTcSmem = size_t(4) * kTcTile * 32 * sizeof(float);

__device__ __forceinline__ bool tile_update_tf32x3(const float* __restrict__ A, int64_t lda,
                                                   const float* __restrict__ B, int64_t ldb, float* __restrict__ C,
                                                   int64_t ldc, int i0, int j0, int mrows, int ncols, int kb,
                                                   float* smem, uint64_t* bar, uint32_t* tslot) {
  float* Ah = smem;
  float* Al = smem + kTcTile * 32;
  float* Bh = smem + 2 * kTcTile * 32;
  float* Bl = smem + 3 * kTcTile * 32;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tmem_alloc(tslot, kTcTile);
  if (tid == 0) mbar_init(bar, 1);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tslot;
  constexpr uint32_t idesc = idesc_tf32(kTcTile, kTcTile);
  bool ok = true;
  for (int h = 0; h < 2 && 32 * h < kb; ++h) {
    const int kbeg = 32 * h;
    {  // A: thread t stages row t of the tile, four K values per 16-byte store (coalesced along the rows)
      const int i = i0 + tid;
      for (int kq = 0; kq < 8; ++kq) {
        float4 h4, l4;
        float* hp = &h4.x;
        float* lp = &l4.x;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int kk = kbeg + 4 * kq + q;
          const float x = (kk < kb && i < mrows) ? A[i + int64_t(kk) * lda] : 0.f;
          split_tf32(x, hp[q], lp[q]);
        }
        const uint32_t o = kmajor_offset(tid, 4 * kq, 32) >> 2;
        *reinterpret_cast<float4*>(Ah + o) = h4;
        *reinterpret_cast<float4*>(Al + o) = l4;
      }
    }
    {  // B: lane l takes column n = 8 r + (l % 8) and K values 4 (l / 8) + 16 s .. +3 of it
      for (int task = warp; task < (kTcTile / 8) * 2; task += kTcThreads / 32) {
        const int n = 8 * (task >> 1) + (lane & 7), kq = (lane >> 3) + 4 * (task & 1);
        const int j = j0 + n;
        float4 h4, l4;
        float* hp = &h4.x;
        float* lp = &l4.x;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int kk = kbeg + 4 * kq + q;
          const float x = (kk < kb && j < ncols) ? B[kk + int64_t(j) * ldb] : 0.f;
          split_tf32(x, hp[q], lp[q]);
        }
        const uint32_t o = kmajor_offset(n, 4 * kq, 32) >> 2;
        *reinterpret_cast<float4*>(Bh + o) = h4;
        *reinterpret_cast<float4*>(Bl + o) = l4;
      }
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
      for (int s = 0; s < 4; ++s) {  // K = 8 per MMA: two core matrices along K
        const uint32_t ks = uint32_t(s) * 256;
        const uint64_t ah = smem_desc(smem_addr(Ah) + ks, 128, 1024), al = smem_desc(smem_addr(Al) + ks, 128, 1024);
        const uint64_t bh = smem_desc(smem_addr(Bh) + ks, 128, 1024), bl = smem_desc(smem_addr(Bl) + ks, 128, 1024);
        mma_tf32(tmem, ah, bh, idesc, (h > 0 || s > 0) ? 1u : 0u);
        mma_tf32(tmem, ah, bl, idesc, 1u);
        mma_tf32(tmem, al, bh, idesc, 1u);
      }
      mma_commit(bar);
    }
    ok = mbar_wait(bar, uint32_t(h & 1)) && ok;
    fence_after_sync();
    __syncthreads();  // the next half overwrites the operands the MMAs read
  }
  const int i = i0 + 32 * warp + lane;
  for (int c = 0; c < kTcTile; c += 16) {
    float v[16];
    tmem_ld16(tmem + (uint32_t(32 * warp) << 16) + uint32_t(c), v);
    if (ok && i < mrows)
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int j = j0 + c + q;
        if (j < ncols) C[i + int64_t(j) * ldc] -= v[q];
      }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTcTile);
  return ok;
}

}  // namespace tc
}  // namespace mgpu
