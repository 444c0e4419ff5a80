// Host symbolic analysis: ordering, elimination tree, column counts,
// relaxed supernodes and the supernodal row structure.  Each step produces
// the same arrays as the reference pipeline it names, so that the numeric
// phase on the GPU works on an identical supernode structure.
#include "symbolic.hpp"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstring>

#include "metis_api.h"

namespace nqg {

using clk = std::chrono::steady_clock;

void sym_permute(const Csc &A, const std::vector<int> &pinv, Csc *lower, Csc *upper) {
  // Two counting passes: bucket entries by their new lower column c, then
  // scatter into upper columns (by new row r) in increasing c, which leaves
  // every upper column sorted; transposing back gives sorted lower columns.
  const int n = A.n;
  const bool vals = !A.x.empty();
  const int64_t nnz = A.nnz();
  std::vector<int> r_of(nnz), c_of(nnz);
  std::vector<int64_t> cnt(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int64_t k = A.p[j]; k < A.p[j + 1]; ++k) {
      int ii = A.i[k];
      if (ii < j) continue;  // only the lower part of a lower-stored matrix counts
      int r = pinv.empty() ? ii : pinv[ii];
      int c = pinv.empty() ? j : pinv[j];
      if (r < c) std::swap(r, c);
      r_of[k] = r;
      c_of[k] = c;
      cnt[r + 1]++;
    }
  // upper: column r holds rows c.  Fill in increasing c by first sorting the
  // entries by c (counting sort).
  std::vector<int64_t> cc(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int64_t k = A.p[j]; k < A.p[j + 1]; ++k)
      if (A.i[k] >= j) cc[c_of[k] + 1]++;
  for (int j = 0; j < n; ++j) cc[j + 1] += cc[j];
  std::vector<int64_t> byc(cc[n]);
  {
    std::vector<int64_t> pos(cc.begin(), cc.end() - 1);
    for (int j = 0; j < n; ++j)
      for (int64_t k = A.p[j]; k < A.p[j + 1]; ++k)
        if (A.i[k] >= j) byc[pos[c_of[k]]++] = k;
  }
  Csc U;
  U.n = n;
  U.p.assign(n + 1, 0);
  for (int j = 0; j < n; ++j) U.p[j + 1] = U.p[j] + (int)cnt[j + 1];
  U.i.resize(U.p[n]);
  if (vals) U.x.resize(U.p[n]);
  {
    std::vector<int> pos(U.p.begin(), U.p.end() - 1);
    for (int64_t t = 0; t < (int64_t)byc.size(); ++t) {
      int64_t k = byc[t];
      int q = pos[r_of[k]]++;
      U.i[q] = c_of[k];
      if (vals) U.x[q] = A.x[k];
    }
  }
  if (lower) {
    Csc Lw;
    Lw.n = n;
    Lw.p.assign(n + 1, 0);
    for (int r = 0; r < n; ++r)
      for (int q = U.p[r]; q < U.p[r + 1]; ++q) Lw.p[U.i[q] + 1]++;
    for (int j = 0; j < n; ++j) Lw.p[j + 1] += Lw.p[j];
    Lw.i.resize(Lw.p[n]);
    if (vals) Lw.x.resize(Lw.p[n]);
    std::vector<int> pos(Lw.p.begin(), Lw.p.end() - 1);
    for (int r = 0; r < n; ++r)
      for (int q = U.p[r]; q < U.p[r + 1]; ++q) {
        int d = pos[U.i[q]]++;
        Lw.i[d] = r;
        if (vals) Lw.x[d] = U.x[q];
      }
    *lower = std::move(Lw);
  }
  if (upper) *upper = std::move(U);
}

// Elimination tree of the matrix whose upper part is `U` (Liu's algorithm
// with path compression; reference etreeC, src/common/Etree.cpp:32).
static void etree_upper(const Csc &U, std::vector<int> &parent) {
  const int n = U.n;
  parent.assign(n, -1);
  std::vector<int> anc(n, -1);
  for (int j = 0; j < n; ++j)
    for (int q = U.p[j]; q < U.p[j + 1]; ++q) {
      int i = U.i[q];
      if (i >= j) continue;
      // climb from i towards the root, compressing the path onto j
      while (true) {
        int a = anc[i];
        if (a == j) break;
        anc[i] = j;
        if (a == -1) {
          parent[i] = j;
          break;
        }
        i = a;
      }
    }
}

// Postorder of a forest (reference postOrderC, src/common/PostOrder.cpp:13):
// roots in increasing index; children visited in increasing index, or, when
// `weight` is given, by increasing weight clamped to [0,n-1] with ties by
// increasing index.
static void postorder(const std::vector<int> &parent, const int *weight, std::vector<int> &post) {
  const int n = (int)parent.size();
  std::vector<int> head(n, -1), next(n, -1);
  if (!weight) {
    for (int j = n - 1; j >= 0; --j) {
      int p = parent[j];
      if (p >= 0 && p < n) {
        next[j] = head[p];
        head[p] = j;
      }
    }
  } else {
    // bucket by weight, then push into parent lists from the heaviest bucket
    // down so that the lightest child (lowest index on ties) ends up first.
    std::vector<int> whead(n, -1), wnext(n, -1);
    for (int j = 0; j < n; ++j) {
      int p = parent[j];
      if (p >= 0 && p < n) {
        int w = std::min(std::max(weight[j], 0), n - 1);
        wnext[j] = whead[w];
        whead[w] = j;
      }
    }
    for (int w = n - 1; w >= 0; --w)
      for (int j = whead[w]; j != -1; j = wnext[j]) {
        int p = parent[j];
        next[j] = head[p];
        head[p] = j;
      }
  }
  post.assign(n, 0);
  std::vector<int> stack(n);
  int k = 0;
  for (int r = 0; r < n; ++r) {
    if (parent[r] != -1) continue;
    int top = 0;
    stack[0] = r;
    while (top >= 0) {
      int p = stack[top];
      int c = head[p];
      if (c == -1) {
        --top;
        post[k++] = p;
      } else {
        head[p] = next[c];
        stack[++top] = c;
      }
    }
  }
}

// Column counts of the Cholesky factor via row-subtree leaves and least
// common ancestors (Gilbert, Ng and Peyton, 1994), from the lower pattern F.
static void column_counts(const Csc &F, const std::vector<int> &parent, const std::vector<int> &post,
                          std::vector<int> &count) {
  const int n = F.n;
  std::vector<int> first(n, -1), maxfirst(n, -1), prevleaf(n, -1), anc(n);
  count.assign(n, 0);
  std::vector<int> &delta = count;
  for (int k = 0; k < n; ++k) {
    int j = post[k];
    delta[j] = (first[j] == -1) ? 1 : 0;
    for (; j != -1 && first[j] == -1; j = parent[j]) first[j] = k;
  }
  for (int i = 0; i < n; ++i) anc[i] = i;
  for (int k = 0; k < n; ++k) {
    int j = post[k];
    if (parent[j] != -1) delta[parent[j]]--;
    for (int q = F.p[j]; q < F.p[j + 1]; ++q) {
      int i = F.i[q];
      if (i <= j || first[j] <= maxfirst[i]) continue;  // j is not a leaf of row i's subtree
      maxfirst[i] = first[j];
      int jprev = prevleaf[i];
      prevleaf[i] = j;
      delta[j]++;
      if (jprev != -1) {
        int lca = jprev;
        while (lca != anc[lca]) lca = anc[lca];
        for (int s = jprev; s != lca;) {
          int sp = anc[s];
          anc[s] = lca;
          s = sp;
        }
        delta[lca]--;
      }
    }
    if (parent[j] != -1) anc[j] = parent[j];
  }
  for (int j = 0; j < n; ++j)
    if (parent[j] != -1) count[parent[j]] += count[j];
}

// Fundamental + relaxed supernodes and their row structure (reference
// super_node_detection, src/symbolic/supernode_detection.cpp:43-746).
static std::string supernodes(const Csc &U, const std::vector<int> &parent, const std::vector<int> &colcount,
                              const std::vector<int> &extra, const int nrelax[3], const double zrelax[3],
                              Symbolic &S) {
  const int n = U.n;
  std::vector<int> nchild(n, 0);
  for (int j = 0; j < n; ++j)
    if (parent[j] != -1) nchild[parent[j]]++;
  std::vector<int> fsuper;
  std::vector<char> single;  // per fundamental supernode: never merged
  fsuper.reserve(n + 1);
  if (n > 0) {
    fsuper.push_back(0);
    single.push_back(0);
  }
  for (int j = 1; j < n; ++j) {
    bool ex = extra[j] == 1 || extra[j - 1] == 1;
    if (parent[j - 1] != j || colcount[j - 1] != colcount[j] + 1 || nchild[j] > 1 || ex) {
      fsuper.push_back(j);
      single.push_back(ex ? 1 : 0);
    }
  }
  const int nf = (int)fsuper.size();
  fsuper.push_back(n);
  std::vector<int> smap(n);
  for (int s = 0; s < nf; ++s)
    for (int k = fsuper[s]; k < fsuper[s + 1]; ++k) smap[k] = s;
  std::vector<int> fparent(nf);
  for (int s = 0; s < nf; ++s) {
    int pj = parent[fsuper[s + 1] - 1];
    fparent[s] = pj == -1 ? -1 : smap[pj];
  }
  std::vector<int> merged(nf, -1), nscol(nf), zeros(nf, 0), snz(nf);
  for (int s = 0; s < nf; ++s) {
    nscol[s] = fsuper[s + 1] - fsuper[s];
    snz[s] = colcount[fsuper[s]];
  }
  for (int s = nf - 2; s >= 0; --s) {
    if (fparent[s] == -1) continue;
    if (single[s] || single[s + 1]) continue;
    int cur = fparent[s];
    while (merged[cur] != -1) cur = merged[cur];
    for (int t = fparent[s]; merged[t] != -1;) {  // path compression
      int nx = merged[t];
      merged[t] = cur;
      t = nx;
    }
    if (cur != s + 1) continue;
    int nc0 = nscol[s], nc1 = nscol[s + 1], ns = nc0 + nc1;
    int totzeros = zeros[s + 1];
    double lnz1 = (double)snz[s + 1];
    bool merge;
    if (ns <= nrelax[0]) {
      merge = true;
    } else {
      double lnz0 = snz[s];
      double xnew = nc0 * (lnz1 + nc0 - lnz0);
      int newzeros = nc0 * (snz[s + 1] + nc0 - snz[s]);
      if (xnew == 0) {
        merge = true;
      } else {
        double xtot = (double)totzeros + xnew;
        double xns = (double)ns;
        double xtotsize = (xns * (xns + 1) / 2) + xns * (lnz1 - nc1);
        double z = xtot / xtotsize;
        totzeros += newzeros;
        merge = ((ns <= nrelax[1] && z < zrelax[0]) || (ns <= nrelax[2] && z < zrelax[1]) || (z < zrelax[2])) &&
                (xtotsize < (double)(INT_MAX / sizeof(double)));
      }
    }
    if (merge) {
      zeros[s] = totzeros;
      merged[s + 1] = s;
      snz[s] = nc0 + snz[s + 1];
      nscol[s] += nscol[s + 1];
    }
  }
  // relaxed supernode list
  S.super.clear();
  std::vector<int> rsnz;
  for (int s = 0; s < nf; ++s)
    if (merged[s] == -1) {
      S.super.push_back(fsuper[s]);
      rsnz.push_back(snz[s]);
    }
  S.nsuper = (int)rsnz.size();
  S.super.push_back(n);
  const int ns = S.nsuper;
  S.col2sup.assign(n, 0);
  for (int s = 0; s < ns; ++s)
    for (int k = S.super[s]; k < S.super[s + 1]; ++k) S.col2sup[k] = s;
  S.sparent.assign(ns, -1);
  for (int s = 0; s < ns; ++s) {
    int pj = parent[S.super[s + 1] - 1];
    S.sparent[s] = pj == -1 ? -1 : S.col2sup[pj];
  }
  // row structure: for every column k of supernode s, walk the supernodal
  // tree upwards from the supernode of every entry i < first(s) of U(:,k),
  // appending k to each supernode reached for the first time for this k.
  S.lpi.assign(ns + 1, 0);
  for (int s = 0; s < ns; ++s) S.lpi[s + 1] = S.lpi[s] + rsnz[s];
  S.ls.assign(std::max<int64_t>(1, S.lpi[ns]), 0);
  std::vector<int64_t> fill(S.lpi.begin(), S.lpi.end() - 1);
  std::vector<int> flag(ns, -1);
  int mark = 0;
  for (int s = 0; s < ns; ++s) {
    int k1 = S.super[s], k2 = S.super[s + 1];
    for (int k = k1; k < k2; ++k) S.ls[fill[s]++] = k;
    for (int k = k1; k < k2; ++k) {
      ++mark;
      flag[s] = mark;
      for (int q = U.p[k]; q < U.p[k + 1]; ++q) {
        int i = U.i[q];
        if (i >= k1) break;  // U columns are sorted
        for (int si = S.col2sup[i]; flag[si] < mark; si = S.sparent[si]) {
          if (fill[si] >= S.lpi[si + 1]) return "supernode row structure overflow";
          S.ls[fill[si]++] = k;
          flag[si] = mark;
        }
      }
    }
  }
  for (int s = 0; s < ns; ++s)
    if (fill[s] != S.lpi[s + 1]) return "supernode row structure does not match its column counts";
  return "";
}

std::string analyze(const Csc &A, const int *extra_cols, const int nrelax[3], const double zrelax[3], Symbolic &S) {
  auto t0 = clk::now();
  const int n = A.n;
  S = Symbolic();
  S.n = n;
  // ---- fill-reducing ordering: METIS nested dissection on the graph of
  // A + A^T without the diagonal.  The adjacency of vertex i lists the
  // strictly-upper entries of column i (i.e. row i of the lower part) first,
  // then the strictly-lower entries of column i, both in increasing order, as
  // the reference builds it (src/symbolic/symbolic_phase.cpp:436-476).
  Csc At;  // upper-stored transpose of A (rows of A)
  {
    std::vector<int> id;
    sym_permute(A, id, nullptr, &At);
  }
  std::vector<int64_t> xadj(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    int64_t cnt = (int64_t)(At.p[i + 1] - At.p[i] - 1) + (int64_t)(A.p[i + 1] - A.p[i] - 1);
    xadj[i + 1] = xadj[i] + cnt;
  }
  std::vector<int64_t> adj(std::max<int64_t>(1, xadj[n]));
  for (int i = 0; i < n; ++i) {
    int64_t b = xadj[i];
    int64_t k = 0;
    for (int q = At.p[i]; q < At.p[i + 1] - 1; ++q) adj[b + k++] = At.i[q];
    for (int q = A.p[i] + 1; q < A.p[i + 1]; ++q) adj[b + k++] = A.i[q];
  }
  std::vector<int64_t> mperm(n), miperm(n);
  {
    int64_t opts[64];
    for (int t = 0; t < 64; ++t) opts[t] = -1;
    METIS_SetDefaultOptions(opts);
    int64_t nv = n;
    auto tm = clk::now();
    int rc = n > 0 ? METIS_NodeND(&nv, xadj.data(), adj.data(), nullptr, opts, mperm.data(), miperm.data()) : 1;
    S.metis_seconds = std::chrono::duration<double>(clk::now() - tm).count();
    if (rc != 1) return "METIS_NodeND failed with code " + std::to_string(rc);
  }
  std::vector<int> perm(n);
  for (int k = 0; k < n; ++k) perm[k] = (int)mperm[k];
  std::vector<int> pinv(n);
  for (int k = 0; k < n; ++k) pinv[perm[k]] = k;

  // ---- etree, postorder and column counts of P A P^T
  Csc Fl, Su;  // lower and upper patterns of the permuted matrix
  {
    Csc Ap = A;
    Ap.x.clear();
    sym_permute(Ap, pinv, &Fl, &Su);
  }
  std::vector<int> parent, post, colcount;
  etree_upper(Su, parent);
  postorder(parent, nullptr, post);
  column_counts(Fl, parent, post, colcount);

  // ---- weighted postorder (weights = column counts), combined with perm
  std::vector<int> wpost;
  postorder(parent, colcount.data(), wpost);
  {
    std::vector<int> np(n), ncc(n), invpost(n), npar(n);
    for (int k = 0; k < n; ++k) {
      np[k] = perm[wpost[k]];
      ncc[k] = colcount[wpost[k]];
      invpost[wpost[k]] = k;
    }
    for (int k = 0; k < n; ++k) {
      int op = parent[wpost[k]];
      npar[k] = op == -1 ? -1 : invpost[op];
    }
    perm.swap(np);
    colcount.swap(ncc);
    parent.swap(npar);
  }
  S.perm = perm;
  S.iperm.assign(n, 0);
  for (int k = 0; k < n; ++k) S.iperm[perm[k]] = k;
  S.parent = parent;
  S.colcount = colcount;
  S.extra_cols.assign(n, 0);
  if (extra_cols)
    for (int k = 0; k < n; ++k) S.extra_cols[k] = extra_cols[perm[k]];

  // ---- supernodes on the final ordering
  Csc U2;
  {
    Csc Ap = A;
    Ap.x.clear();
    sym_permute(Ap, S.iperm, nullptr, &U2);
  }
  std::string err = supernodes(U2, parent, colcount, S.extra_cols, nrelax, zrelax, S);
  if (!err.empty()) return err;

  // ---- value layout: each supernode is a dense column-major nrow x ncol
  // block, leading dimension nrow, columns contiguous (reference L->p).
  const int ns = S.nsuper;
  S.lpx.assign(ns + 1, 0);
  S.colp.assign(n + 1, 0);
  S.max_sup_wid = 0;
  S.max_col = 0;
  for (int s = 0; s < ns; ++s) {
    int w = S.super[s + 1] - S.super[s];
    int64_t r = S.lpi[s + 1] - S.lpi[s];
    S.max_sup_wid = std::max(S.max_sup_wid, w);
    S.max_col = std::max<int>(S.max_col, (int)r);
    S.lpx[s + 1] = S.lpx[s] + r * w;
    for (int c = 0; c < w; ++c) S.colp[S.super[s] + c] = S.lpx[s] + (int64_t)c * r;
  }
  if (n > 0) S.colp[n] = S.lpx[ns];
  S.xsize = std::max<int64_t>(1, S.lpx[ns]);
  S.total_seconds = std::chrono::duration<double>(clk::now() - t0).count();
  return "";
}

void ereach_sn(const Symbolic &S, const Csc &U, int s, const std::vector<int> &tree, std::vector<int> &mark,
               std::vector<int> &stack, std::vector<int> &out) {
  // Supernodes reached from the entries of U(0:first(s)-1, cols of s),
  // climbing `tree` until a marked node; a node whose tree entry is -2
  // (hidden) stops the climb.  Output is in the reference's stack order.
  const int ns = S.nsuper;
  int c1 = S.super[s], c2 = S.super[s + 1];
  out.clear();
  stack.resize(ns);
  int top = ns;
  std::vector<int> path;
  mark[s] = 1;
  for (int k = c1; k < c2; ++k)
    for (int q = U.p[k]; q < U.p[k + 1]; ++q) {
      int r = U.i[q];
      if (r > k) continue;
      int i = S.col2sup[r];
      path.clear();
      while (i >= 0 && !mark[i] && tree[i] != -2) {
        path.push_back(i);
        mark[i] = 1;
        i = tree[i];
      }
      for (int t = (int)path.size() - 1; t >= 0; --t) stack[--top] = path[t];
    }
  for (int t = top; t < ns; ++t) {
    out.push_back(stack[t]);
    mark[stack[t]] = 0;
  }
  mark[s] = 0;
}

}  // namespace nqg
