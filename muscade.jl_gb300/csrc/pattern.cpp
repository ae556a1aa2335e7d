// Sparsity pattern and scatter plans (see pattern.hpp).
#include "pattern.hpp"

#include <algorithm>
#include <cstdio>

namespace mgpu {

std::string build_pattern(int64_t n, const std::vector<GroupShape>& groups, Pattern& P) {
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
    for (int64_t k = 0; k < G.nele * G.nX; ++k) {
      const int64_t d = G.indexX[k];
      if (d < 1 || d > n) return "dof index out of range in indexX";
    }
  }
  if (kb >= (int64_t(1) << 32) || rb >= (int64_t(1) << 32)) return "model too large for 32-bit scatter plans";
  P.kbuf_size = kb;
  P.rbuf_size = rb;

  // ---- bucket the pairs by column j (stable in pair order)
  std::vector<int64_t> cstart(n + 1, 0);
  for (size_t g = 0; g < ng; ++g) {
    const GroupShape& G = groups[g];
    for (int64_t e = 0; e < G.nele; ++e)
      for (int j = 0; j < G.nX; ++j) cstart[G.indexX[e * G.nX + j]] += G.nX;
  }
  for (int64_t j = 0; j < n; ++j) cstart[j + 1] += cstart[j];
  std::vector<int32_t> crow(npair);
  std::vector<uint32_t> csrc(npair);   // kbuf offset of the pair
  std::vector<int64_t> cpair(npair);   // pair id
  {
    std::vector<int64_t> fill(cstart.begin(), cstart.end() - 1);
    for (size_t g = 0; g < ng; ++g) {
      const GroupShape& G = groups[g];
      const int nX = G.nX;
      for (int64_t e = 0; e < G.nele; ++e) {
        const int64_t* ix = G.indexX + e * nX;
        for (int j = 0; j < nX; ++j) {
          const int64_t col = ix[j] - 1;
          for (int i = 0; i < nX; ++i) {
            const int64_t pos = fill[col]++;
            const int64_t entry = i + int64_t(nX) * j;
            crow[pos] = int32_t(ix[i] - 1);
            csrc[pos] = uint32_t(P.kbuf_base[g] + entry * G.nele + e);
            cpair[pos] = P.pair_base[g] + e * nX * nX + entry;
          }
        }
      }
    }
  }
  // ---- per column: order by row (stable, keeps pair order), count distinct rows
  std::vector<int64_t> cnnz(n, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t j = 0; j < n; ++j) {
    const int64_t a = cstart[j], b = cstart[j + 1];
    if (b - a > 1) {
      std::vector<int64_t> ord(b - a);
      for (int64_t k = 0; k < b - a; ++k) ord[k] = a + k;
      std::stable_sort(ord.begin(), ord.end(), [&](int64_t x, int64_t y) { return crow[x] < crow[y]; });
      std::vector<int32_t> r2(b - a);
      std::vector<uint32_t> s2(b - a);
      std::vector<int64_t> p2(b - a);
      for (int64_t k = 0; k < b - a; ++k) {
        r2[k] = crow[ord[k]];
        s2[k] = csrc[ord[k]];
        p2[k] = cpair[ord[k]];
      }
      std::copy(r2.begin(), r2.end(), crow.begin() + a);
      std::copy(s2.begin(), s2.end(), csrc.begin() + a);
      std::copy(p2.begin(), p2.end(), cpair.begin() + a);
    }
    int64_t c = 0;
    for (int64_t k = a; k < b; ++k)
      if (k == a || crow[k] != crow[k - 1]) ++c;
    cnnz[j] = c;
  }
  P.colptr.assign(n + 1, 0);
  for (int64_t j = 0; j < n; ++j) P.colptr[j + 1] = P.colptr[j] + cnnz[j];
  P.nnz = P.colptr[n];
  if (P.nnz >= (int64_t(1) << 31)) return "too many nonzeros";
  P.rowval.resize(P.nnz);
  P.pair_nnz.resize(npair);
  P.mseg.resize(P.nnz + 1);
  P.msrc.resize(npair);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t j = 0; j < n; ++j) {
    int64_t k = P.colptr[j] - 1;
    for (int64_t q = cstart[j]; q < cstart[j + 1]; ++q) {
      if (q == cstart[j] || crow[q] != crow[q - 1]) {
        ++k;
        P.rowval[k] = crow[q];
        P.mseg[k] = uint32_t(q);  // sources of nnz k start at q (columns are contiguous in q)
      }
      P.pair_nnz[cpair[q]] = int32_t(k);
      P.msrc[q] = csrc[q];
    }
  }
  P.mseg[P.nnz] = uint32_t(npair);

  // ---- vector plan: sources of each dof in pair order (type, element, entry)
  P.vseg.assign(n + 1, 0);
  std::vector<int64_t> vcount(n + 1, 0);
  for (size_t g = 0; g < ng; ++g) {
    const GroupShape& G = groups[g];
    for (int64_t k = 0; k < G.nele * G.nX; ++k) vcount[G.indexX[k]] += 1;
  }
  for (int64_t i = 0; i < n; ++i) vcount[i + 1] += vcount[i];
  for (int64_t i = 0; i <= n; ++i) P.vseg[i] = uint32_t(vcount[i]);
  P.vsrc.resize(vcount[n]);
  {
    std::vector<int64_t> fill(vcount.begin(), vcount.end() - 1);
    for (size_t g = 0; g < ng; ++g) {
      const GroupShape& G = groups[g];
      for (int64_t e = 0; e < G.nele; ++e)
        for (int i = 0; i < G.nX; ++i) {
          const int64_t d = G.indexX[e * G.nX + i] - 1;
          P.vsrc[fill[d]++] = uint32_t(P.rbuf_base[g] + int64_t(i) * G.nele + e);
        }
    }
  }
  return "";
}

}  // namespace mgpu
