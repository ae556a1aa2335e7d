// Host harness of the sparse solver's analysis (muscade.jl_gb300/csrc/sparse_analysis.cpp),
// compiled with g++ by tests/test_sparse_analysis.py so that the ordering,
// the symbolic factorisation and the assembly maps are checked on the CPU.
#include <cstring>

#include "../muscade.jl_gb300/csrc/sparse_analysis.hpp"

using namespace mgpu;

struct Handle {
  SparseAnalysis A;
  std::string err;
};

extern "C" {

void* sh_analyse(int64_t n, const int64_t* colptr, const int32_t* rowval, const double* xyz, const uint8_t* last,
                 int leaf) {
  Handle* h = new Handle();
  SparseInput in;
  in.n = n;
  in.colptr = colptr;
  in.rowval = rowval;
  in.xyz = xyz;
  in.last = last;
  in.leaf_groups = leaf;
  h->err = sparse_analyse(in, h->A);
  return h;
}

const char* sh_error(void* p) { return static_cast<Handle*>(p)->err.c_str(); }

// nfronts, len(fidx), len(emap), fsize, nheight, max_children, ngroups, max_m
void sh_sizes(void* p, int64_t* s) {
  const SparseAnalysis& A = static_cast<Handle*>(p)->A;
  s[0] = int64_t(A.fronts.size());
  s[1] = int64_t(A.fidx.size());
  s[2] = int64_t(A.emap.size());
  s[3] = A.fsize;
  s[4] = A.nheight;
  s[5] = A.max_children;
  s[6] = A.ngroups;
  s[7] = A.max_m;
}

// fronts[nf][9] = off, idx, eoff, m, p, pos0, parent, height, crank
void sh_get(void* p, int32_t* perm, int64_t* fronts, int32_t* fidx, int32_t* emap, int64_t* amap, double* flops) {
  const SparseAnalysis& A = static_cast<Handle*>(p)->A;
  std::memcpy(perm, A.perm.data(), A.perm.size() * sizeof(int32_t));
  for (size_t f = 0; f < A.fronts.size(); ++f) {
    const SparseFront& F = A.fronts[f];
    int64_t* r = fronts + 9 * f;
    r[0] = F.off;
    r[1] = F.idx;
    r[2] = F.eoff;
    r[3] = F.m;
    r[4] = F.p;
    r[5] = F.pos0;
    r[6] = F.parent;
    r[7] = F.height;
    r[8] = F.crank;
  }
  std::memcpy(fidx, A.fidx.data(), A.fidx.size() * sizeof(int32_t));
  std::memcpy(emap, A.emap.data(), A.emap.size() * sizeof(int32_t));
  std::memcpy(amap, A.amap.data(), A.amap.size() * sizeof(int64_t));
  *flops = A.flops;
}

void sh_free(void* p) { delete static_cast<Handle*>(p); }
}
