// The CSC pattern of Lλx and its gather plan built on the device (the same
// result as build_pattern in pattern.cpp, which restates asmmat!,
// src/Assemble.jl:373-448).  Every element entry (j, i) of every element is a
// pair with key j·n + i and id (element type, element, i + nX·j) in the
// reference's accumulation order.  A stable least-significant-digit radix
// sort of the keys (8-bit digits, ids carried along) leaves the pairs of one
// nonzero together and in id order; the heads of equal-key runs number the
// nonzeros.  From the sorted pairs: rowval and colptr, the nonzero of every
// pair (asm2), and the plan of the gather (the first sorted position of each
// nonzero and the element-entry buffer offset of each sorted pair).  The
// vector plan (one entry per element dof) stays on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "pattern.hpp"

namespace mgpu {
namespace {

constexpr int kRsThreads = 256;
constexpr int kRsPer = 16;                       // keys per thread and tile
constexpr int kRsTile = kRsThreads * kRsPer;     // keys per block
constexpr int kRsDigits = 256;

struct GroupDev {
  int64_t nele, pair_base, kbuf_base;
  int32_t nX;
  const int32_t* idx;  // [nX][nele] 0-based
};

// keys and ids of the pairs of one group (ids in pair order)
__global__ void pd_pairs(GroupDev G, int64_t n, uint64_t* __restrict__ key, uint32_t* __restrict__ id) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t np = G.nele * G.nX * G.nX;
  if (q >= np) return;
  const int nX = G.nX;
  const int64_t e = q / (nX * nX);
  const int ent = int(q % (nX * nX));
  const int i = ent % nX, j = ent / nX;
  const int64_t row = G.idx[int64_t(i) * G.nele + e], col = G.idx[int64_t(j) * G.nele + e];
  key[G.pair_base + q] = uint64_t(col) * uint64_t(n) + uint64_t(row);
  id[G.pair_base + q] = uint32_t(G.pair_base + q);
}

// per tile: the count of each digit
__global__ void __launch_bounds__(kRsThreads) pd_hist(int64_t m, const uint64_t* __restrict__ key, int shift,
                                                      uint32_t* __restrict__ counts, int64_t ntile) {
  __shared__ uint32_t h[kRsDigits];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = int64_t(blockIdx.x) * kRsTile;
  for (int u = 0; u < kRsPer; ++u) {
    const int64_t q = base + int64_t(u) * kRsThreads + threadIdx.x;
    if (q < m) atomicAdd(&h[(key[q] >> shift) & 0xFF], 1u);
  }
  __syncthreads();
  counts[int64_t(threadIdx.x) * ntile + blockIdx.x] = h[threadIdx.x];  // digit-major
}

// exclusive scan of cnt elements in place, one block walking the array in
// chunks (used for the per-chunk totals of the multi-block scan below)
__global__ void __launch_bounds__(1024) pd_scan(int64_t cnt, uint32_t* __restrict__ a) {
  __shared__ uint32_t s[1024];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t c0 = 0; c0 < cnt; c0 += 1024) {
    const int64_t q = c0 + threadIdx.x;
    const uint32_t v = q < cnt ? a[q] : 0u;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {  // inclusive Hillis-Steele
      const uint32_t t = threadIdx.x >= d ? s[threadIdx.x - d] : 0u;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (q < cnt) a[q] = carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += s[1023];
    __syncthreads();
  }
}

// multi-block exclusive scan: each block scans a chunk of kScanChunk elements
// (kScanPer consecutive ones per thread) and leaves the chunk's total in
// sums; pd_scan turns the totals into offsets and pd_scan_add adds them
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 8;
constexpr int64_t kScanChunk = int64_t(kScanThreads) * kScanPer;

__global__ void __launch_bounds__(kScanThreads) pd_scan_chunk(int64_t cnt, uint32_t* __restrict__ a,
                                                              uint32_t* __restrict__ sums) {
  __shared__ uint32_t s[kScanThreads];
  const int64_t base = int64_t(blockIdx.x) * kScanChunk + int64_t(threadIdx.x) * kScanPer;
  uint32_t v[kScanPer], run = 0;
#pragma unroll
  for (int u = 0; u < kScanPer; ++u) {
    v[u] = base + u < cnt ? a[base + u] : 0u;
    run += v[u];
  }
  s[threadIdx.x] = run;
  __syncthreads();
  for (int d = 1; d < kScanThreads; d <<= 1) {
    const uint32_t t = threadIdx.x >= d ? s[threadIdx.x - d] : 0u;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  uint32_t off = s[threadIdx.x] - run;
#pragma unroll
  for (int u = 0; u < kScanPer; ++u) {
    if (base + u < cnt) a[base + u] = off;
    off += v[u];
  }
  if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void __launch_bounds__(kScanThreads) pd_scan_add(int64_t cnt, uint32_t* __restrict__ a,
                                                            const uint32_t* __restrict__ sums) {
  const uint32_t add = sums[blockIdx.x];
  const int64_t base = int64_t(blockIdx.x) * kScanChunk;
  for (int u = 0; u < kScanPer; ++u) {
    const int64_t q = base + int64_t(u) * kScanThreads + threadIdx.x;
    if (q < cnt) a[q] += add;
  }
}

// exclusive scan of cnt elements of a (sums: one entry per chunk)
void scan(int64_t cnt, uint32_t* a, uint32_t* sums, cudaStream_t st) {
  const int64_t nb = (cnt + kScanChunk - 1) / kScanChunk;
  if (nb <= 0) return;
  pd_scan_chunk<<<unsigned(nb), kScanThreads, 0, st>>>(cnt, a, sums);
  pd_scan<<<1, 1024, 0, st>>>(nb, sums);
  pd_scan_add<<<unsigned(nb), kScanThreads, 0, st>>>(cnt, a, sums);
}

// stable scatter of one tile: a key's destination is its digit's offset for
// the tile plus the number of keys with that digit before it in the tile
__global__ void __launch_bounds__(kRsThreads) pd_scatter(int64_t m, const uint64_t* __restrict__ key,
                                                         const uint32_t* __restrict__ id, int shift,
                                                         const uint32_t* __restrict__ offs, int64_t ntile,
                                                         uint64_t* __restrict__ key2, uint32_t* __restrict__ id2) {
  constexpr int NW = kRsThreads / 32;
  __shared__ uint32_t base[kRsDigits];
  __shared__ uint32_t wcnt[NW][kRsDigits];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  base[tid] = offs[int64_t(tid) * ntile + blockIdx.x];
  const int64_t t0 = int64_t(blockIdx.x) * kRsTile;
  for (int u = 0; u < kRsPer; ++u) {
    for (int w = 0; w < NW; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const int64_t q = t0 + int64_t(u) * kRsThreads + tid;
    const bool valid = q < m;
    const uint64_t k = valid ? key[q] : 0;
    const uint32_t dg = valid ? uint32_t((k >> shift) & 0xFF) : 0xFFFFFFFFu;
    const unsigned peers = __match_any_sync(0xffffffffu, dg);
    const unsigned lower = peers & ((1u << lane) - 1u);
    const int rank_w = __popc(lower);
    if (valid && lower == 0) wcnt[warp][dg] = __popc(peers);  // the first lane of the digit group
    __syncthreads();
    if (valid) {
      uint32_t before = 0;
      for (int w = 0; w < warp; ++w) before += wcnt[w][dg];
      const uint32_t dst = base[dg] + before + uint32_t(rank_w);
      key2[dst] = k;
      id2[dst] = id[q];
    }
    __syncthreads();
    uint32_t tot = 0;  // this chunk's count of digit tid
    for (int w = 0; w < NW; ++w) tot += wcnt[w][tid];
    base[tid] += tot;
    __syncthreads();
  }
}

// heads of equal-key runs (1) in sorted order
__global__ void pd_heads(int64_t m, const uint64_t* __restrict__ key, uint32_t* __restrict__ head) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q < m) head[q] = (q == 0 || key[q] != key[q - 1]) ? 1u : 0u;
}

// with hs the exclusive scan of the heads: nonzero k = hs[q] − 1 + head;
// rowval, column counts, the plan's segment starts and sources, and asm2
__global__ void pd_emit(int64_t m, int64_t n, const uint64_t* __restrict__ key, const uint32_t* __restrict__ id,
                        const uint32_t* __restrict__ hs, const uint32_t* __restrict__ head,
                        const GroupDev* __restrict__ groups, int ngroup, int32_t* __restrict__ rowval,
                        uint32_t* __restrict__ colcnt, uint32_t* __restrict__ mseg, uint32_t* __restrict__ msrc,
                        int32_t* __restrict__ pair_nnz) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= m) return;
  const uint32_t k = hs[q] + head[q] - 1u;
  const uint32_t pid = id[q];
  if (head[q]) {
    rowval[k] = int32_t(key[q] % uint64_t(n));
    atomicAdd(&colcnt[key[q] / uint64_t(n)], 1u);
    mseg[k] = uint32_t(q);
  }
  int g = 0;
  while (g + 1 < ngroup && int64_t(pid) >= groups[g + 1].pair_base) ++g;
  const GroupDev G = groups[g];
  const int64_t r = int64_t(pid) - G.pair_base;
  const int64_t e = r / (G.nX * G.nX);
  const int64_t ent = r % (G.nX * G.nX);
  msrc[q] = uint32_t(G.kbuf_base + ent * G.nele + e);
  pair_nnz[pid] = int32_t(k);
}

}  // namespace

std::string build_pattern_device(int64_t n, const std::vector<GroupShape>& groups,
                                 const std::vector<const int32_t*>& d_idx, cudaStream_t st, Pattern& P) {
  // shapes, bases and the vector plan as on the host
  P = Pattern();
  P.n = n;
  const size_t ng = groups.size();
  P.pair_base.resize(ng);
  P.kbuf_base.resize(ng);
  P.rbuf_base.resize(ng);
  int64_t npair = 0, kb = 0, rb = 0;
  for (size_t g = 0; g < ng; ++g) {
    const GroupShape& G = groups[g];
    if (G.nX < 0 || G.nele < 0) return "invalid element group shape";
    P.pair_base[g] = npair;
    P.kbuf_base[g] = kb;
    P.rbuf_base[g] = rb;
    npair += G.nele * G.nX * G.nX;
    kb += G.nele * G.nX * G.nX;
    rb += G.nele * G.nX;
    for (int64_t k = 0; k < G.nele * G.nX; ++k)
      if (G.indexX[k] < 1 || G.indexX[k] > n) return "dof index out of range in indexX";
  }
  if (kb >= (int64_t(1) << 32) || rb >= (int64_t(1) << 32)) return "model too large for 32-bit scatter plans";
  P.kbuf_size = kb;
  P.rbuf_size = rb;
  {
    std::vector<int64_t> vcount(n + 1, 0);
    for (size_t g = 0; g < ng; ++g)
      for (int64_t k = 0; k < groups[g].nele * groups[g].nX; ++k) vcount[groups[g].indexX[k]] += 1;
    for (int64_t i = 0; i < n; ++i) vcount[i + 1] += vcount[i];
    P.vseg.assign(n + 1, 0);
    for (int64_t i = 0; i <= n; ++i) P.vseg[i] = uint32_t(vcount[i]);
    P.vsrc.resize(vcount[n]);
    std::vector<int64_t> fill(vcount.begin(), vcount.end() - 1);
    for (size_t g = 0; g < ng; ++g) {
      const GroupShape& G = groups[g];
      for (int64_t e = 0; e < G.nele; ++e)
        for (int i = 0; i < G.nX; ++i)
          P.vsrc[fill[G.indexX[e * G.nX + i] - 1]++] = uint32_t(P.rbuf_base[g] + int64_t(i) * G.nele + e);
    }
  }
  const int64_t m = npair;
  P.colptr.assign(n + 1, 0);
  P.mseg.assign(1, 0);
  if (m == 0) {
    P.nnz = 0;
    return "";
  }
  // device work
  std::vector<void*> owned;
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    for (void* p : owned) cudaFree(p);
  };
  auto dal = [&](auto** p, size_t cnt) -> bool {
    if (cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(cnt, 1) * sizeof(**p)) != cudaSuccess) return false;
    owned.push_back(*p);
    return true;
  };
  const int64_t ntile = (m + kRsTile - 1) / kRsTile;
  uint64_t *k1, *k2;
  uint32_t *i1, *i2, *counts, *head, *hs, *colcnt, *mseg, *msrc, *sums;
  int32_t *rowval, *pnnz;
  GroupDev* dgroups;
  if (!dal(&k1, m) || !dal(&k2, m) || !dal(&i1, m) || !dal(&i2, m) || !dal(&counts, size_t(kRsDigits) * ntile) ||
      !dal(&head, m) || !dal(&hs, m) || !dal(&colcnt, n + 1) || !dal(&mseg, m) || !dal(&msrc, m) ||
      !dal(&rowval, m) || !dal(&pnnz, m) || !dal(&dgroups, ng) ||
      !dal(&sums, size_t(std::max<int64_t>(int64_t(kRsDigits) * ntile, m) / kScanChunk + 1))) {
    cleanup();
    return "device pattern: allocation failed";
  }
  std::vector<GroupDev> hg(ng);
  for (size_t g = 0; g < ng; ++g)
    hg[g] = GroupDev{groups[g].nele, P.pair_base[g], P.kbuf_base[g], groups[g].nX, d_idx[g]};
  cudaError_t e = cudaMemcpyAsync(dgroups, hg.data(), ng * sizeof(GroupDev), cudaMemcpyHostToDevice, st);
  for (size_t g = 0; g < ng && e == cudaSuccess; ++g) {
    const int64_t np = groups[g].nele * groups[g].nX * groups[g].nX;
    if (np > 0) pd_pairs<<<unsigned((np + 255) / 256), 256, 0, st>>>(hg[g], n, k1, i1);
  }
  int bits = 1;
  while (bits < 64 && (uint64_t(1) << bits) < uint64_t(n) * uint64_t(n)) ++bits;
  for (int shift = 0; shift < bits && e == cudaSuccess; shift += 8) {
    pd_hist<<<unsigned(ntile), kRsThreads, 0, st>>>(m, k1, shift, counts, ntile);
    scan(int64_t(kRsDigits) * ntile, counts, sums, st);
    pd_scatter<<<unsigned(ntile), kRsThreads, 0, st>>>(m, k1, i1, shift, counts, ntile, k2, i2);
    std::swap(k1, k2);
    std::swap(i1, i2);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    pd_heads<<<unsigned((m + 255) / 256), 256, 0, st>>>(m, k1, head);
    e = cudaMemcpyAsync(hs, head, m * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
  }
  if (e == cudaSuccess) {
    // an exclusive scan of the heads (in chunks of the counts scan) and the emission
    scan(m, hs, sums, st);
    e = cudaMemsetAsync(colcnt, 0, (n + 1) * sizeof(uint32_t), st);
  }
  if (e == cudaSuccess) {
    pd_emit<<<unsigned((m + 255) / 256), 256, 0, st>>>(m, n, k1, i1, hs, head, dgroups, int(ng), rowval, colcnt, mseg,
                                                       msrc, pnnz);
    e = cudaGetLastError();
  }
  uint32_t last_hs = 0, last_head = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&last_hs, hs + m - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&last_head, head + m - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    const std::string msg = std::string("device pattern: ") + cudaGetErrorString(e);
    cleanup();
    return msg;
  }
  const int64_t nnz = int64_t(last_hs) + last_head;
  if (nnz >= (int64_t(1) << 31)) {
    cleanup();
    return "too many nonzeros";
  }
  P.nnz = nnz;
  P.rowval.resize(nnz);
  P.pair_nnz.resize(m);
  P.mseg.resize(nnz + 1);
  P.msrc.resize(m);
  std::vector<uint32_t> cc(n + 1);
  e = cudaMemcpyAsync(P.rowval.data(), rowval, nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(P.pair_nnz.data(), pnnz, m * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(P.mseg.data(), mseg, nnz * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(P.msrc.data(), msrc, m * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cc.data(), colcnt, (n + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) return std::string("device pattern: ") + cudaGetErrorString(e);
  P.mseg[nnz] = uint32_t(m);
  for (int64_t j = 0; j < n; ++j) P.colptr[j + 1] = P.colptr[j] + cc[j];
  return "";
}

}  // namespace mgpu
