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
// C[i0 .. i0+128) × [j0 .. j0+128) −= A[·, kbeg..kend) · B[kbeg..kend, ·], with
// A(i, k) = A[i + k·lda], B(k, j) = B[k + j·ldb], C(i, j) = C[i + j·ldc], rows
// below mrows and columns below ncols.  Each operand is split as x = hi + lo
// (hi its TF32 rounding) and the accumulator takes Aₕ·Bₕ + Aₕ·Bₗ + Aₗ·Bₕ.
// K runs in chunks of kTcKc through two shared-memory stages: the threads load
// chunk c + 1 into registers while the MMAs of chunk c run, and overwrite a
// stage only after the MMAs of its previous chunk have completed (one
// mbarrier per stage, bounded waits).  128 threads; smem: kTcSmem bytes,
// 128-byte aligned; bar[2], tslot: shared.  Warp 0 holds 128 tensor-memory
// columns for the 128 × 128 FP32 accumulator (row i in lane i) and frees them
// before returning.  Returns false when the MMAs did not complete within the
// bounded waits (then C is left unchanged).
constexpr int kTcTile = 128;
constexpr int kTcThreads = 128;
constexpr int kTcKc = 16;                                 // K per stage
constexpr int kTcOperand = kTcTile * kTcKc;               // floats of one split operand of a stage
constexpr int kTcStage = 4 * kTcOperand;                  // Aₕ, Aₗ, Bₕ, Bₗ
constexpr size_t kTcSmem = size_t(2) * kTcStage * sizeof(float);
constexpr int64_t kTcPolls = int64_t(1) << 20;  // bound of one wait (a chunk's MMAs take well under a microsecond)

// one chunk's operands in registers: A row `tid` (kTcKc values) and, for B,
// lane l's k-quad (l >> 3) of column 8·task + (l & 7) for the warp's four tasks
struct TcChunk {
  float a[kTcKc];
  float b[kTcKc];
};

__device__ __forceinline__ void tc_load_chunk(TcChunk& v, const float* __restrict__ A, int64_t lda,
                                              const float* __restrict__ B, int64_t ldb, int i0, int j0, int mrows,
                                              int ncols, int kc, int kend) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i = i0 + tid;
#pragma unroll
  for (int k = 0; k < kTcKc; ++k) {
    const int kk = kc + k;
    v.a[k] = (kk < kend && i < mrows) ? A[i + int64_t(kk) * lda] : 0.f;
  }
#pragma unroll
  for (int tt = 0; tt < 4; ++tt) {
    const int task = warp + 4 * tt;
    const int j = j0 + 8 * task + (lane & 7), kq = lane >> 3;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int kk = kc + 4 * kq + q;
      v.b[4 * tt + q] = (kk < kend && j < ncols) ? B[kk + int64_t(j) * ldb] : 0.f;
    }
  }
}

// split and store one chunk in the canonical K-major layout (16-byte stores,
// a warp's 32 stores covering 512 contiguous bytes)
__device__ __forceinline__ void tc_store_chunk(const TcChunk& v, float* Ah, float* Al, float* Bh, float* Bl) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
#pragma unroll
  for (int kq = 0; kq < kTcKc / 4; ++kq) {
    float4 h4, l4;
    split_tf32(v.a[4 * kq + 0], h4.x, l4.x);
    split_tf32(v.a[4 * kq + 1], h4.y, l4.y);
    split_tf32(v.a[4 * kq + 2], h4.z, l4.z);
    split_tf32(v.a[4 * kq + 3], h4.w, l4.w);
    const uint32_t o = kmajor_offset(tid, 4 * kq, kTcKc) >> 2;
    *reinterpret_cast<float4*>(Ah + o) = h4;
    *reinterpret_cast<float4*>(Al + o) = l4;
  }
#pragma unroll
  for (int tt = 0; tt < 4; ++tt) {
    const int task = warp + 4 * tt;
    const int n = 8 * task + (lane & 7), kq = lane >> 3;
    float4 h4, l4;
    split_tf32(v.b[4 * tt + 0], h4.x, l4.x);
    split_tf32(v.b[4 * tt + 1], h4.y, l4.y);
    split_tf32(v.b[4 * tt + 2], h4.z, l4.z);
    split_tf32(v.b[4 * tt + 3], h4.w, l4.w);
    const uint32_t o = kmajor_offset(n, 4 * kq, kTcKc) >> 2;
    *reinterpret_cast<float4*>(Bh + o) = h4;
    *reinterpret_cast<float4*>(Bl + o) = l4;
  }
}

// one chunk through its stage: wait until the stage's previous chunk has been
// consumed (block-uniform outcome), split and store, one thread issues the
// six MMAs and commits them to the stage's mbarrier
__device__ __forceinline__ bool tc_chunk_mma(const TcChunk& v, int c, float* smem, uint64_t* bar, uint32_t tmem) {
  const int tid = threadIdx.x;
  const int s = c & 1;
  float* Ah = smem + s * kTcStage;
  float* Al = Ah + kTcOperand;
  float* Bh = Al + kTcOperand;
  float* Bl = Bh + kTcOperand;
  if (c >= 2 && !__syncthreads_and(mbar_wait(bar + s, uint32_t(((c - 2) >> 1) & 1), kTcPolls) ? 1 : 0)) return false;
  tc_store_chunk(v, Ah, Al, Bh, Bl);
  fence_async_smem();
  __syncthreads();
  if (tid == 0) {
    fence_after_sync();
    constexpr uint32_t idesc = idesc_tf32(kTcTile, kTcTile);
    constexpr uint32_t kLbo = 128, kSbo = (kTcKc / 4) * 128;  // core matrices along K, along M/N
#pragma unroll
    for (int ks = 0; ks < kTcKc / 8; ++ks) {  // K = 8 per MMA: two core matrices along K
      const uint32_t off = uint32_t(ks) * 256;
      const uint64_t ah = smem_desc(smem_addr(Ah) + off, kLbo, kSbo), al = smem_desc(smem_addr(Al) + off, kLbo, kSbo);
      const uint64_t bh = smem_desc(smem_addr(Bh) + off, kLbo, kSbo), bl = smem_desc(smem_addr(Bl) + off, kLbo, kSbo);
      mma_tf32(tmem, ah, bh, idesc, (c > 0 || ks > 0) ? 1u : 0u);
      mma_tf32(tmem, ah, bl, idesc, 1u);
      mma_tf32(tmem, al, bh, idesc, 1u);
    }
    mma_commit(bar + s);
  }
  return true;
}

__device__ __forceinline__ bool tile_update_tf32x3(const float* __restrict__ A, int64_t lda,
                                                   const float* __restrict__ B, int64_t ldb, float* __restrict__ C,
                                                   int64_t ldc, int i0, int j0, int mrows, int ncols, int kbeg,
                                                   int kend, float* smem, uint64_t* bar, uint32_t* tslot) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nch = (kend - kbeg + kTcKc - 1) / kTcKc;
  // the loads of two chunks in flight: chunk c + 2 is loaded once chunk c is stored
  TcChunk v0, v1;
  tc_load_chunk(v0, A, lda, B, ldb, i0, j0, mrows, ncols, kbeg, kend);
  if (nch > 1) tc_load_chunk(v1, A, lda, B, ldb, i0, j0, mrows, ncols, kbeg + kTcKc, kend);
  if (warp == 0) {
    tmem_alloc(tslot, kTcTile);
    tmem_relinquish();  // lets the SM's other blocks allocate while this one runs
  }
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init(bar + 1, 1);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tslot;
  bool ok = true;
#pragma unroll 1
  for (int c = 0; c < nch && ok; c += 2) {
    ok = tc_chunk_mma(v0, c, smem, bar, tmem);
    if (!ok) break;
    if (c + 2 < nch) tc_load_chunk(v0, A, lda, B, ldb, i0, j0, mrows, ncols, kbeg + (c + 2) * kTcKc, kend);
    if (c + 1 < nch) {
      ok = tc_chunk_mma(v1, c + 1, smem, bar, tmem);
      if (!ok) break;
      if (c + 3 < nch) tc_load_chunk(v1, A, lda, B, ldb, i0, j0, mrows, ncols, kbeg + (c + 3) * kTcKc, kend);
    }
  }
  // the last chunk's commit arrives once every MMA of the tile has completed
  if (ok && nch > 0)
    ok = __syncthreads_and(mbar_wait(bar + ((nch - 1) & 1), uint32_t(((nch - 1) >> 1) & 1), kTcPolls) ? 1 : 0) != 0;
  fence_after_sync();
  // epilogue: 32 accumulator columns at a time, their C loads all in flight together
  const int i = i0 + 32 * warp + lane;
  const bool row_ok = ok && nch > 0 && i < mrows;
  for (int c = 0; c < kTcTile; c += 32) {
    float v0[16], v1[16];
    tmem_ld16(tmem + (uint32_t(32 * warp) << 16) + uint32_t(c), v0);
    tmem_ld16(tmem + (uint32_t(32 * warp) << 16) + uint32_t(c + 16), v1);
    float cv[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int j = j0 + c + q;
      cv[q] = (row_ok && j < ncols) ? C[i + int64_t(j) * ldc] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int j = j0 + c + q;
      if (row_ok && j < ncols) C[i + int64_t(j) * ldc] = cv[q] - (q < 16 ? v0[q] : v1[q - 16]);
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTcTile);
  return ok;
}

}  // namespace tc
}  // namespace mgpu
