// Host analysis of the sparse direct solver (see sparse_analysis.hpp).
#include "sparse_analysis.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <unordered_map>

namespace mgpu {
namespace {

using Graph = std::vector<std::vector<int32_t>>;  // sorted adjacency lists, no self loops

uint64_t mix(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

struct UnionFind {
  std::vector<int32_t> p;
  explicit UnionFind(size_t n) : p(n) { std::iota(p.begin(), p.end(), 0); }
  int32_t find(int32_t a) {
    while (p[a] != a) {
      p[a] = p[p[a]];
      a = p[a];
    }
    return a;
  }
  void unite(int32_t a, int32_t b) {
    a = find(a);
    b = find(b);
    if (a != b) p[std::max(a, b)] = std::min(a, b);
  }
};

// vertices with equal closed neighbourhoods N[v] = adj(v) ∪ {v} are merged
void merge_indistinguishable(const Graph& G, UnionFind& uf) {
  const size_t n = G.size();
  std::vector<std::pair<uint64_t, int32_t>> key(n);
  for (size_t v = 0; v < n; ++v) {
    uint64_t h = mix(uint64_t(v));
    for (int32_t w : G[v]) h += mix(uint64_t(w));
    key[v] = {h ^ (uint64_t(G[v].size()) << 1), int32_t(v)};
  }
  std::sort(key.begin(), key.end());
  auto closed_equal = [&](int32_t a, int32_t b) {
    // N[a] == N[b]: a ∈ adj(b), b ∈ adj(a) and adj(a) \ {b} == adj(b) \ {a}
    const auto& A = G[a];
    const auto& B = G[b];
    if (A.size() != B.size()) return false;
    size_t i = 0, j = 0;
    bool ab = false, ba = false;
    while (i < A.size() || j < B.size()) {
      if (i < A.size() && A[i] == b) {
        ab = true;
        ++i;
        continue;
      }
      if (j < B.size() && B[j] == a) {
        ba = true;
        ++j;
        continue;
      }
      if (i >= A.size() || j >= B.size() || A[i] != B[j]) return false;
      ++i;
      ++j;
    }
    return ab && ba;
  };
  for (size_t s = 0; s < n;) {
    size_t e = s + 1;
    while (e < n && key[e].first == key[s].first) ++e;
    for (size_t a = s; a < e; ++a)
      for (size_t b = a + 1; b < e; ++b)
        if (uf.find(key[a].second) != uf.find(key[b].second) && closed_equal(key[a].second, key[b].second))
          uf.unite(key[a].second, key[b].second);
    s = e;
  }
}

// quotient graph of the groups of uf over G; grp[v] = group index of vertex v
Graph quotient(const Graph& G, UnionFind& uf, std::vector<int32_t>& grp, int32_t& ng) {
  const size_t n = G.size();
  std::vector<int32_t> id(n, -1);
  ng = 0;
  grp.assign(n, -1);
  for (size_t v = 0; v < n; ++v) {
    const int32_t r = uf.find(int32_t(v));
    if (id[r] < 0) id[r] = ng++;
    grp[v] = id[r];
  }
  Graph Q(ng);
  for (size_t v = 0; v < n; ++v)
    for (int32_t w : G[v])
      if (grp[w] != grp[v]) Q[grp[v]].push_back(grp[w]);
  for (auto& a : Q) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  return Q;
}

struct NDBuilder {
  const Graph& G;                  // group graph
  const std::vector<double>& xyz;  // [ng][3]
  int leaf;
  std::vector<int32_t> mark;       // per group: id of the part it currently belongs to
  int32_t stamp = 0;
  struct Node {
    std::vector<int32_t> groups;
    std::vector<int32_t> children;
  };
  std::vector<Node> nodes;  // in postorder
  NDBuilder(const Graph& g, const std::vector<double>& c, int lf) : G(g), xyz(c), leaf(lf), mark(g.size(), -1) {}

  int32_t emit(std::vector<int32_t> groups, std::vector<int32_t> children) {
    nodes.push_back(Node{std::move(groups), std::move(children)});
    return int32_t(nodes.size() - 1);
  }

  // connected components of the vertex set V (induced subgraph)
  std::vector<std::vector<int32_t>> components(const std::vector<int32_t>& V) {
    const int32_t s = ++stamp;
    for (int32_t v : V) mark[v] = s;
    std::vector<std::vector<int32_t>> out;
    const int32_t done = ++stamp;
    for (int32_t v0 : V) {
      if (mark[v0] != s) continue;
      std::vector<int32_t> comp{v0};
      mark[v0] = done;
      for (size_t h = 0; h < comp.size(); ++h)
        for (int32_t w : G[comp[h]])
          if (mark[w] == s) {
            mark[w] = done;
            comp.push_back(w);
          }
      out.push_back(std::move(comp));
    }
    return out;
  }

  // roots of the subtrees that eliminate V
  std::vector<int32_t> dissect(std::vector<int32_t> V) {
    if (V.empty()) return {};
    if (int(V.size()) <= leaf) {
      std::sort(V.begin(), V.end());
      return {emit(std::move(V), {})};
    }
    auto comps = components(V);
    if (comps.size() > 1) {
      std::vector<int32_t> roots;
      for (auto& cpt : comps) {
        auto r = dissect(std::move(cpt));
        roots.insert(roots.end(), r.begin(), r.end());
      }
      return roots;
    }
    // split at the median of the longest coordinate extent
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int32_t v : V)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], xyz[3 * v + d]);
        hi[d] = std::max(hi[d], xyz[3 * v + d]);
      }
    int ax = 0;
    for (int d = 1; d < 3; ++d)
      if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
    std::vector<double> cv(V.size());
    for (size_t k = 0; k < V.size(); ++k) cv[k] = xyz[3 * V[k] + ax];
    std::vector<double> sorted = cv;
    std::nth_element(sorted.begin(), sorted.begin() + sorted.size() / 2, sorted.end());
    const double med = sorted[sorted.size() / 2];
    std::vector<int32_t> A, B;
    for (size_t k = 0; k < V.size(); ++k) (cv[k] < med ? A : B).push_back(V[k]);
    if (A.empty() || B.empty()) {  // no spread along the axis: split in vertex order
      A.clear();
      B.clear();
      std::sort(V.begin(), V.end());
      A.assign(V.begin(), V.begin() + V.size() / 2);
      B.assign(V.begin() + V.size() / 2, V.end());
    }
    // vertex separator: the vertices of one side that touch the other; take the smaller
    const int32_t sa = ++stamp;
    for (int32_t v : A) mark[v] = sa;
    const int32_t sb = ++stamp;
    for (int32_t v : B) mark[v] = sb;
    std::vector<int32_t> SA, SB, A2, B2;
    for (int32_t v : A) {
      bool t = false;
      for (int32_t w : G[v]) t |= mark[w] == sb;
      (t ? SA : A2).push_back(v);
    }
    for (int32_t v : B) {
      bool t = false;
      for (int32_t w : G[v]) t |= mark[w] == sa;
      (t ? SB : B2).push_back(v);
    }
    std::vector<int32_t> S;
    if (SB.size() <= SA.size()) {
      S = std::move(SB);
      B = std::move(B2);
    } else {
      S = std::move(SA);
      A = std::move(A2);
    }
    auto ra = dissect(std::move(A));
    auto rb = dissect(std::move(B));
    ra.insert(ra.end(), rb.begin(), rb.end());
    std::sort(S.begin(), S.end());
    return {emit(std::move(S), std::move(ra))};
  }
};

}  // namespace

std::string sparse_analyse(const SparseInput& in, SparseAnalysis& out) {
  out = SparseAnalysis();
  const int64_t n = in.n;
  if (n <= 0) return "empty matrix";
  if (n >= (int64_t(1) << 31)) return "matrix too large";
  out.n = n;
  out.nnz = in.colptr[n];
  // ---- dof graph (symmetrised pattern without the diagonal)
  Graph D(n);
  out.diag.assign(n, -1);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t q = in.colptr[j]; q < in.colptr[j + 1]; ++q) {
      const int32_t i = in.rowval[q];
      if (i == j) {
        out.diag[j] = int32_t(q);
        continue;
      }
      D[j].push_back(i);
      D[i].push_back(int32_t(j));
    }
  for (auto& a : D) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  // ---- compression: dofs of a node; multipliers join the dof they constrain
  UnionFind uf(n);
  merge_indistinguishable(D, uf);
  std::vector<int32_t> grp;
  int32_t ng = 0;
  for (int round = 0; round < 3; ++round) {
    Graph Q = quotient(D, uf, grp, ng);
    // a group with one neighbour group joins it
    std::vector<int32_t> rep(ng, -1);  // a dof of each group
    for (int64_t v = 0; v < n; ++v)
      if (rep[grp[v]] < 0) rep[grp[v]] = int32_t(v);
    bool changed = false;
    for (int32_t g = 0; g < ng; ++g)
      if (Q[g].size() == 1) {
        uf.unite(rep[g], rep[Q[g][0]]);
        changed = true;
      }
    Q = quotient(D, uf, grp, ng);
    // groups with equal closed neighbourhoods in the group graph
    UnionFind ug(ng);
    merge_indistinguishable(Q, ug);
    std::vector<int32_t> rep2(ng, -1);
    for (int64_t v = 0; v < n; ++v)
      if (rep2[grp[v]] < 0) rep2[grp[v]] = int32_t(v);
    for (int32_t g = 0; g < ng; ++g)
      if (ug.find(g) != g) {
        uf.unite(rep2[g], rep2[ug.find(g)]);
        changed = true;
      }
    if (!changed) break;
  }
  Graph Q = quotient(D, uf, grp, ng);
  out.ngroups = ng;
  std::vector<std::vector<int32_t>> members(ng);
  for (int64_t v = 0; v < n; ++v) members[grp[v]].push_back(int32_t(v));
  for (auto& M : members)  // dofs in increasing order, constraint multipliers last
    std::stable_partition(M.begin(), M.end(), [&](int32_t v) { return !(in.last && in.last[v]); });
  // ---- group coordinates: mean of the members' known coordinates, else of the neighbours'
  std::vector<double> gx(3 * size_t(ng), 0.0);
  std::vector<uint8_t> known(ng, 0);
  if (in.xyz)
    for (int32_t g = 0; g < ng; ++g) {
      int cnt = 0;
      double s[3] = {0, 0, 0};
      for (int32_t v : members[g])
        if (std::isfinite(in.xyz[3 * v]) && std::isfinite(in.xyz[3 * v + 1]) && std::isfinite(in.xyz[3 * v + 2])) {
          for (int d = 0; d < 3; ++d) s[d] += in.xyz[3 * v + d];
          ++cnt;
        }
      if (cnt) {
        for (int d = 0; d < 3; ++d) gx[3 * g + d] = s[d] / cnt;
        known[g] = 1;
      }
    }
  for (int sweep = 0; sweep < 64; ++sweep) {
    bool any = false;
    std::vector<uint8_t> k2 = known;
    for (int32_t g = 0; g < ng; ++g) {
      if (known[g]) continue;
      int cnt = 0;
      double s[3] = {0, 0, 0};
      for (int32_t h : Q[g])
        if (known[h]) {
          for (int d = 0; d < 3; ++d) s[d] += gx[3 * h + d];
          ++cnt;
        }
      if (cnt) {
        for (int d = 0; d < 3; ++d) gx[3 * g + d] = s[d] / cnt;
        k2[g] = 1;
        any = true;
      }
    }
    known.swap(k2);
    if (!any) break;
  }
  // ---- nested dissection of the group graph
  NDBuilder nd(Q, gx, std::max(1, in.leaf_groups));
  {
    std::vector<int32_t> all(ng);
    std::iota(all.begin(), all.end(), 0);
    nd.dissect(std::move(all));
  }
  const int32_t nf = int32_t(nd.nodes.size());
  // ---- elimination positions, in postorder of the dissection tree
  out.perm.resize(n);
  out.ipos.assign(n, -1);
  out.fronts.resize(nf);
  std::vector<int32_t> gpos0(ng, -1);
  {
    int32_t pos = 0;
    for (int32_t f = 0; f < nf; ++f) {
      SparseFront& F = out.fronts[f];
      F.pos0 = pos;
      for (int32_t g : nd.nodes[f].groups) {
        gpos0[g] = pos;
        for (int32_t v : members[g]) {
          out.perm[pos] = v;
          out.ipos[v] = pos++;
        }
      }
      F.p = pos - F.pos0;
      for (size_t c = 0; c < nd.nodes[f].children.size(); ++c) {
        SparseFront& C = out.fronts[nd.nodes[f].children[c]];
        C.parent = f;
        C.crank = int32_t(c);
      }
      out.max_children = std::max<int>(out.max_children, int(nd.nodes[f].children.size()));
    }
    if (pos != n) return "nested dissection lost dofs";
  }
  // ---- symbolic factorisation on the group graph: update groups of each front
  std::vector<std::vector<int32_t>> upd(nf);  // groups, sorted by elimination position
  {
    std::vector<int32_t> seen(ng, -1);
    for (int32_t f = 0; f < nf; ++f) {
      const int32_t end = out.fronts[f].pos0 + out.fronts[f].p;
      std::vector<int32_t>& U = upd[f];
      for (int32_t g : nd.nodes[f].groups)
        for (int32_t h : Q[g])
          if (gpos0[h] >= end && seen[h] != f) {
            seen[h] = f;
            U.push_back(h);
          }
      for (int32_t c : nd.nodes[f].children) {
        for (int32_t h : upd[c])
          if (gpos0[h] >= end && seen[h] != f) {
            seen[h] = f;
            U.push_back(h);
          }
      }
      std::sort(U.begin(), U.end(), [&](int32_t a, int32_t b) { return gpos0[a] < gpos0[b]; });
    }
  }
  // ---- index lists, heights, layout
  std::vector<int64_t> idx0(nf);
  {
    int64_t t = 0;
    for (int32_t f = 0; f < nf; ++f) {
      SparseFront& F = out.fronts[f];
      int64_t m = F.p;
      for (int32_t h : upd[f]) m += int64_t(members[h].size());
      if (m >= (int64_t(1) << 31) / 2) return "front too large";
      F.m = int32_t(m);
      F.idx = t;
      idx0[f] = t;
      t += m;
      out.max_m = std::max(out.max_m, F.m);
      out.max_p = std::max(out.max_p, F.p);
    }
    out.fidx.resize(t);
    for (int32_t f = 0; f < nf; ++f) {
      const SparseFront& F = out.fronts[f];
      int64_t k = F.idx;
      for (int32_t i = 0; i < F.p; ++i) out.fidx[k++] = F.pos0 + i;
      for (int32_t h : upd[f])
        for (size_t i = 0; i < members[h].size(); ++i) out.fidx[k++] = gpos0[h] + int32_t(i);
    }
    for (int32_t f = 0; f < nf; ++f) {
      int32_t h = 0;
      for (int32_t c : nd.nodes[f].children) h = std::max(h, out.fronts[c].height + 1);
      out.fronts[f].height = h;
      out.nheight = std::max(out.nheight, h + 1);
    }
    std::vector<int32_t> byh(nf);
    std::iota(byh.begin(), byh.end(), 0);
    std::stable_sort(byh.begin(), byh.end(),
                     [&](int32_t a, int32_t b) { return out.fronts[a].height < out.fronts[b].height; });
    int64_t off = 0;
    for (int32_t f : byh) {
      out.fronts[f].off = off;
      off += int64_t(out.fronts[f].m) * out.fronts[f].m;
    }
    out.fsize = off;
  }
  // local index of an elimination position in front f
  auto local = [&](int32_t f, int32_t pos) -> int32_t {
    const SparseFront& F = out.fronts[f];
    if (pos >= F.pos0 && pos < F.pos0 + F.p) return pos - F.pos0;
    const int32_t* a = out.fidx.data() + F.idx + F.p;
    const int32_t* b = out.fidx.data() + F.idx + F.m;
    const int32_t* it = std::lower_bound(a, b, pos);
    if (it == b || *it != pos) return -1;
    return int32_t(F.p + (it - a));
  };
  // ---- extend-add maps
  {
    int64_t t = 0;
    for (int32_t f = 0; f < nf; ++f)
      if (out.fronts[f].parent >= 0) {
        out.fronts[f].eoff = t;
        t += out.fronts[f].m - out.fronts[f].p;
      }
    out.emap.resize(t);
    for (int32_t f = 0; f < nf; ++f) {
      const SparseFront& F = out.fronts[f];
      if (F.parent < 0) {
        if (F.m != F.p) return "root front with update rows";
        continue;
      }
      for (int32_t k = F.p; k < F.m; ++k) {
        const int32_t l = local(F.parent, out.fidx[F.idx + k]);
        if (l < 0) return "update row missing from the parent front";
        out.emap[F.eoff + (k - F.p)] = l;
      }
    }
  }
  // ---- front of each elimination position, and the place of every nnz
  std::vector<int32_t> fpos(n);
  for (int32_t f = 0; f < nf; ++f)
    for (int32_t i = 0; i < out.fronts[f].p; ++i) fpos[out.fronts[f].pos0 + i] = f;
  out.amap.resize(out.nnz);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t q = in.colptr[j]; q < in.colptr[j + 1]; ++q) {
      const int32_t pi = out.ipos[in.rowval[q]], pj = out.ipos[j];
      const int32_t f = fpos[std::min(pi, pj)];
      const int32_t li = local(f, pi), lj = local(f, pj);
      if (li < 0 || lj < 0) return "matrix entry outside its front";
      out.amap[q] = out.fronts[f].off + int64_t(lj) * out.fronts[f].m + li;
    }
  // ---- flops of the partial factorisations
  for (const SparseFront& F : out.fronts)
    for (int32_t k = 0; k < F.p; ++k) {
      const double r = double(F.m - k - 1);
      out.flops += r + 2.0 * r * r;
    }
  return "";
}

}  // namespace mgpu
