// Host side of the batched QP solver: problem intake, grouping by sparsity
// pattern, one symbolic analysis per pattern (the reference's ordering and
// supernodes, reference SolverSettings::symbolic_analysis,
// src/QP/linear_solver_wrapper.cpp:396-536), the integer work lists of each
// pattern, per-problem values and settings, device layout, the CUDA-graph
// launch of the persistent kernel (batch.cu), and the C ABI
// (include/nasoq_gb300.h, nqg_batch_*).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/nasoq_gb300.h"
#include "batch.hpp"
#include "plan.hpp"
#include "qp_rules.hpp"
#include "symbolic.hpp"

namespace {

using nqg::BPat;
using nqg::BProb;
using nqg::BResult;

struct HostQP {
  int n = 0, meq = 0, mineq = 0;
  std::vector<int> Hp, Hi, Ap, Ai, Cp, Ci;
  std::vector<double> Hx, q, Ax, b, Cx, d;
  int pat = -1;
  std::vector<int> ws;  // proposed active set (warm start)
  bool warm = false;
};

struct HostPattern {
  int rep = -1;  // a problem of this pattern
  BPat P{};
  nqg::Symbolic S;
  // integer arrays of this pattern, in BPat offset order (filled by build_pattern)
  std::vector<int> super, sparent, col2sup, lpi, lpx, ls0, perm0, lvl_ptr, lvl_sn, lev, pair_ptr, pair_mid, pair_d,
      pair_lb, pair_ub, Rp, Rj, Rq, ent, bt_ptr, bt_var, bt_q, bt_rpos, sn_con, con_sn, eq_ptr, eq_var, eq_q,
      snrec, prec, con_ptr, con_tgt, sn_big;
  std::vector<int> diag_q;  // per column: value index of its diagonal
};

uint64_t fnv(uint64_t h, const void *p, size_t bytes) {
  const unsigned char *c = static_cast<const unsigned char *>(p);
  for (size_t k = 0; k < bytes; ++k) {
    h ^= c[k];
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t pattern_key(const HostQP &Q) {
  uint64_t h = 1469598103934665603ull;
  int dims[3] = {Q.n, Q.meq, Q.mineq};
  h = fnv(h, dims, sizeof dims);
  for (const std::vector<int> *v : {&Q.Hp, &Q.Hi, &Q.Ap, &Q.Ai, &Q.Cp, &Q.Ci}) h = fnv(h, v->data(), v->size() * 4);
  return h;
}

bool same_pattern(const HostQP &a, const HostQP &b) {
  return a.n == b.n && a.meq == b.meq && a.mineq == b.mineq && a.Hp == b.Hp && a.Hi == b.Hi && a.Ap == b.Ap &&
         a.Ai == b.Ai && a.Cp == b.Cp && a.Ci == b.Ci;
}

// Lower CSC pattern of the super-KKT [H; A; C] (the reference's
// build_super_matrix: H columns, then the equality rows, then the
// inequality rows; one diagonal entry per constraint column) and, when
// `vals`, the original values with every constraint entry present.
void super_kkt(const HostQP &Q, nqg::Csc &K, std::vector<double> *vals) {
  const int n = Q.n, N = Q.n + Q.meq + Q.mineq, base = Q.n + Q.meq;
  K.n = N;
  K.p.assign(N + 1, 0);
  K.i.clear();
  if (vals) vals->clear();
  for (int j = 0; j < n; ++j) {
    for (int q = Q.Hp[j]; q < Q.Hp[j + 1]; ++q) {
      K.i.push_back(Q.Hi[q]);
      if (vals) vals->push_back(Q.Hx[q]);
    }
    if (Q.meq)
      for (int q = Q.Ap[j]; q < Q.Ap[j + 1]; ++q) {
        K.i.push_back(n + Q.Ai[q]);
        if (vals) vals->push_back(Q.Ax[q]);
      }
    if (Q.mineq)
      for (int q = Q.Cp[j]; q < Q.Cp[j + 1]; ++q) {
        K.i.push_back(base + Q.Ci[q]);
        if (vals) vals->push_back(Q.Cx[q]);
      }
    K.p[j + 1] = (int)K.i.size();
  }
  for (int k = n; k < N; ++k) {
    K.i.push_back(k);
    if (vals) vals->push_back(0.0);
    K.p[k + 1] = (int)K.i.size();
  }
}

std::string build_pattern(const HostQP &Q, HostPattern &H, const int nrelax[3], const double zrelax[3]) {
  const int n = Q.n, meq = Q.meq, mineq = Q.mineq, N = n + meq + mineq, base = n + meq;
  nqg::Csc K;
  super_kkt(Q, K, nullptr);
  std::vector<int> extra(N, 0);
  for (int j = base; j < N; ++j) extra[j] = 1;
  nqg::Symbolic &S = H.S;
  std::string err = nqg::analyze(K, extra.data(), nrelax, zrelax, S);
  if (!err.empty()) return err;
  const int ns = S.nsuper;
  if (S.xsize > (1ll << 30) || (int64_t)S.ls.size() > (1ll << 30)) return "pattern too large for the batched solver";
  BPat &P = H.P;
  P.n = n;
  P.meq = meq;
  P.mineq = mineq;
  P.N = N;
  P.base = base;
  P.ns = ns;
  P.xsize = (int)S.xsize;
  P.ssize = (int)S.ls.size();
  P.nnzK = (int)K.nnz();
  H.super = S.super;
  H.sparent = S.sparent;
  H.col2sup = S.col2sup;
  H.lpi.assign(S.lpi.begin(), S.lpi.end());
  H.lpx.assign(S.lpx.begin(), S.lpx.end());
  H.ls0 = S.ls;
  H.perm0 = S.perm;
  P.max_w = 0;
  P.max_nr = 0;
  for (int s = 0; s < ns; ++s) {
    P.max_w = std::max(P.max_w, S.super[s + 1] - S.super[s]);
    P.max_nr = std::max(P.max_nr, (int)(S.lpi[s + 1] - S.lpi[s]));
  }
  H.sn_con.assign(ns, -1);
  H.con_sn.assign(mineq, -1);
  for (int k = 0; k < mineq; ++k) {
    const int oc = S.iperm[base + k];
    const int s = S.col2sup[oc];
    if (S.super[s + 1] - S.super[s] != 1) return "an inequality column is not a single-column supernode";
    H.con_sn[k] = s;
    H.sn_con[s] = k;
  }
  for (int s = 0; s < ns; ++s)
    if (S.sparent[s] >= 0 && S.sparent[s] <= s) return "supernodes are not numbered in postorder";
  // levels (leaves first)
  std::vector<int> lev(ns, 0);
  int maxl = 0;
  for (int s = 0; s < ns; ++s) {
    const int p = S.sparent[s];
    if (p >= 0) lev[p] = std::max(lev[p], lev[s] + 1);
    maxl = std::max(maxl, lev[s]);
  }
  P.nlev = ns ? maxl + 1 : 0;
  H.lvl_ptr.assign(P.nlev + 1, 0);
  for (int s = 0; s < ns; ++s) H.lvl_ptr[lev[s] + 1]++;
  for (int l = 0; l < P.nlev; ++l) H.lvl_ptr[l + 1] += H.lvl_ptr[l];
  H.lvl_sn.assign(ns, 0);
  {
    std::vector<int> pos(H.lvl_ptr.begin(), H.lvl_ptr.end() - (P.nlev ? 1 : 0));
    for (int s = 0; s < ns; ++s) H.lvl_sn[pos[lev[s]]++] = s;
  }
  H.lev = lev;
  // descendant pairs from the elimination-tree reach (reference ereach_sn)
  nqg::Csc up;
  nqg::sym_permute(K, S.iperm, nullptr, &up);
  std::vector<int> mark(ns, 0), stack, lst;
  H.pair_ptr.assign(ns + 1, 0);
  H.pair_mid.assign(ns, 0);
  for (int s = 0; s < ns; ++s) {
    nqg::ereach_sn(S, up, s, S.sparent, mark, stack, lst);
    // descendants that never hide first, then the constraint columns
    std::stable_partition(lst.begin(), lst.end(), [&](int d) { return H.sn_con[d] < 0; });
    const int c1 = S.super[s], c2 = S.super[s + 1];
    int nstruct = 0;
    for (int d : lst) {
      const int *rows = S.ls.data() + S.lpi[d];
      const int nr = (int)(S.lpi[d + 1] - S.lpi[d]);
      const int lb = (int)(std::lower_bound(rows, rows + nr, c1) - rows);
      const int ub = (int)(std::lower_bound(rows, rows + nr, c2) - rows) - 1;
      if (lb >= nr || ub < lb) continue;
      H.pair_d.push_back(d);
      H.pair_lb.push_back(lb);
      H.pair_ub.push_back(ub);
      if (H.sn_con[d] < 0) nstruct++;
    }
    H.pair_mid[s] = H.pair_ptr[s] + nstruct;
    H.pair_ptr[s + 1] = (int)H.pair_d.size();
  }
  // full symmetric CSR of K in the original numbering, with value indices
  const int nz = (int)K.nnz();
  H.Rp.assign(N + 1, 0);
  for (int j = 0; j < N; ++j)
    for (int q = K.p[j]; q < K.p[j + 1]; ++q) {
      H.Rp[j + 1]++;
      if (K.i[q] != j) H.Rp[K.i[q] + 1]++;
    }
  for (int r = 0; r < N; ++r) H.Rp[r + 1] += H.Rp[r];
  H.Rj.assign(H.Rp[N], 0);
  H.Rq.assign(H.Rp[N], 0);
  {
    std::vector<int> pos(H.Rp.begin(), H.Rp.end() - 1);
    for (int j = 0; j < N; ++j)
      for (int q = K.p[j]; q < K.p[j + 1]; ++q) {
        const int i = K.i[q];
        H.Rj[pos[j]] = i;
        H.Rq[pos[j]++] = q;
        if (i != j) {
          H.Rj[pos[i]] = j;
          H.Rq[pos[i]++] = q;
        }
      }
  }
  // entry kinds, constraint and equality row lists
  H.ent.assign(nz, -1);
  H.diag_q.assign(N, -1);
  std::vector<std::vector<int>> btv(mineq), btq(mineq), eqv(meq), eqq(meq);
  for (int j = 0; j < N; ++j) {
    for (int q = K.p[j]; q < K.p[j + 1]; ++q) {
      const int i = K.i[q];
      if (i == j) {
        H.ent[q] = -2 - j;
        H.diag_q[j] = q;
      } else if (i >= base) {
        H.ent[q] = i - base;
        btv[i - base].push_back(j);
        btq[i - base].push_back(q);
      } else if (i >= n) {
        eqv[i - n].push_back(j);
        eqq[i - n].push_back(q);
      }
    }
    if (H.diag_q[j] != K.p[j]) return "every column of H needs its diagonal entry stored first";
  }
  auto flatten = [](const std::vector<std::vector<int>> &v, const std::vector<std::vector<int>> &w,
                    std::vector<int> &ptr, std::vector<int> &a, std::vector<int> &b) {
    ptr.assign(v.size() + 1, 0);
    for (size_t k = 0; k < v.size(); ++k) {
      ptr[k + 1] = ptr[k] + (int)v[k].size();
      a.insert(a.end(), v[k].begin(), v[k].end());
      b.insert(b.end(), w[k].begin(), w[k].end());
    }
  };
  flatten(btv, btq, H.bt_ptr, H.bt_var, H.bt_q);
  H.bt_rpos.assign(H.bt_var.size(), -1);
  for (int k = 0; k < mineq; ++k)
    for (int e = H.bt_ptr[k]; e < H.bt_ptr[k + 1]; ++e) {
      const int v = H.bt_var[e];
      for (int qq = H.Rp[v]; qq < H.Rp[v + 1]; ++qq)
        if (H.Rj[qq] == base + k) H.bt_rpos[e] = qq;
      if (H.bt_rpos[e] < 0) return "constraint entry missing from the symmetric pattern";
    }
  P.nnzR = H.Rp[N];
  // packed records: one load brings a supernode's or a pair's numbers
  H.snrec.assign((size_t)8 * ns, 0);
  for (int s = 0; s < ns; ++s) {
    int *r = H.snrec.data() + 8 * (size_t)s;
    r[0] = S.super[s];
    r[1] = S.super[s + 1] - S.super[s];
    r[2] = (int)(S.lpi[s + 1] - S.lpi[s]);
    r[3] = (int)S.lpx[s];
    r[4] = (int)S.lpi[s];
    r[5] = H.pair_ptr[s];
    r[6] = H.pair_mid[s];
    r[7] = H.pair_ptr[s + 1];
  }
  const int npairs = (int)H.pair_d.size();
  H.prec.assign((size_t)4 * npairs, 0);
  std::vector<std::vector<int>> ctg(mineq);
  P.cmask_ok = 1;
  for (int s = 0; s < ns; ++s) {
    if (H.pair_ptr[s + 1] - H.pair_mid[s] > 64) P.cmask_ok = 0;
    for (int pq = H.pair_ptr[s]; pq < H.pair_ptr[s + 1]; ++pq) {
      const int d = H.pair_d[pq];
      int *r = H.prec.data() + 4 * (size_t)pq;
      r[0] = d;
      r[1] = H.pair_lb[pq];
      r[2] = H.pair_ub[pq];
      r[3] = (int)S.lpi[d];
      if (pq >= H.pair_mid[s]) {
        const int k = H.sn_con[d];
        ctg[k].push_back(s);
        ctg[k].push_back(pq - H.pair_mid[s]);
      }
    }
  }
  // supernodes the solves give a warp: wide or tall blocks (one flag byte each, packed in ints)
  H.sn_big.assign((ns + 3) / 4 + 1, 0);
  for (int s = 0; s < ns; ++s) {
    const int w = S.super[s + 1] - S.super[s], nr = (int)(S.lpi[s + 1] - S.lpi[s]);
    if (w > 4 || (int64_t)nr * w > 64) reinterpret_cast<unsigned char *>(H.sn_big.data())[s] = 1;
  }
  H.con_ptr.assign(mineq + 1, 0);
  for (int k = 0; k < mineq; ++k) {
    H.con_ptr[k + 1] = H.con_ptr[k] + (int)ctg[k].size() / 2;
    H.con_tgt.insert(H.con_tgt.end(), ctg[k].begin(), ctg[k].end());
  }
  flatten(eqv, eqq, H.eq_ptr, H.eq_var, H.eq_q);
  return "";
}

}  // namespace

struct TierLaunch {
  nqg::BArgs args{};
  size_t smem = 0;
  int grid = 0, bps = 0, nprob = 0, order_off = 0;
  int64_t slot_off = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
};

struct nqg_batch {
  nqg_batch_settings set{};
  std::vector<HostQP> qp;
  std::vector<HostPattern> pats;
  bool finalized = false;
  std::string last_error;
  // device
  cudaStream_t stream = nullptr;
  nqg::BArgs args{};
  BPat *d_pats = nullptr;
  BProb *d_probs = nullptr;
  int *d_ipool = nullptr, *d_order = nullptr, *d_head = nullptr, *d_iout = nullptr;
  double *d_dpool = nullptr, *d_dout = nullptr;
  BResult *d_res = nullptr;
  unsigned char *d_slots = nullptr;
  std::vector<BProb> h_probs;
  std::vector<double> h_dpool;  // doubles part of the value pool (pert bytes follow on the device)
  int64_t n_dbl = 0, n_pert_bytes = 0, n_dout = 0, n_iout = 0;
  int grid = 0, threads = 128, blocks_per_sm = 0, num_sms = 0;
  size_t smem = 0;
  // groups of problems with identical matrices: one shared factorization each
  unsigned char *d_bases = nullptr;
  int *d_base_rep = nullptr;
  int nbase = 0;
  // staging of set_vectors: stacked q / b / d and their offsets per problem
  double *d_vstage = nullptr;
  int64_t *d_voff = nullptr;
  std::vector<int64_t> h_voff;  // segment offsets of the last nqg_batch_set_vectors
  int64_t n_vstage = 0;
  cudaGraphExec_t gexec = nullptr;
  cudaGraph_t graph = nullptr;
  double last_ms = 0.0;
  cudaEvent_t e0 = nullptr, e1 = nullptr, efork = nullptr;
  std::vector<TierLaunch> tiers;
  unsigned long long *d_prof = nullptr;
};

namespace {

int fail(nqg_batch *b, int code, const std::string &msg) {
  b->last_error = msg;
  return code;
}

#define BQ_CUDA(call)                                                             \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) return fail(b, NQG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void free_device(nqg_batch *b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->gexec = nullptr;
  b->graph = nullptr;
  if (b->d_prof) cudaFree(b->d_prof);
  b->d_prof = nullptr;
  for (void *p : {(void *)b->d_pats, (void *)b->d_probs, (void *)b->d_ipool, (void *)b->d_order, (void *)b->d_head,
                  (void *)b->d_iout, (void *)b->d_dpool, (void *)b->d_dout, (void *)b->d_res, (void *)b->d_slots,
                  (void *)b->d_bases, (void *)b->d_base_rep, (void *)b->d_vstage, (void *)b->d_voff})
    if (p) cudaFree(p);
  b->d_bases = nullptr;
  b->d_base_rep = nullptr;
  b->d_vstage = nullptr;
  b->d_voff = nullptr;
  b->d_pats = nullptr;
  b->d_probs = nullptr;
  b->d_ipool = b->d_order = b->d_head = b->d_iout = nullptr;
  b->d_dpool = b->d_dout = nullptr;
  b->d_res = nullptr;
  b->d_slots = nullptr;
}

// Derived settings of one problem (reference Nasoq::symbolic_QP,
// src/nasoq.cpp:222-280): regularization, refinement counts and tolerance
// from the variant.
int problem_settings(const nqg_batch_settings &st, const HostQP &Q, BProb &P) {
  const nqg_qp_settings &s = st.qp;
  double reg = s.diag_perturb, tol = s.stop_tol;
  int outer = s.max_iter, inner = s.max_iter;
  const size_t total_nnz = (size_t)Q.Hp[Q.n] + (size_t)(Q.mineq ? Q.Cp[Q.n] : 0);
  const double H_norm2 = nqg::qp_frob_lower(Q.n, Q.Hp.data(), Q.Hi.data(), Q.Hx.data());
  if (s.variant == 1) {  // AUTO
    nqg::qp_auto_perturbation2(Q.n, total_nnz, H_norm2, 0.0, Q.mineq, Q.mineq / double(Q.n), s.eps_abs, reg, outer,
                               inner, tol);
  } else if (s.variant == 0) {  // Fixed
    nqg::qp_determine_iterations(total_nnz, s.eps_abs, outer, inner);
    tol = 1e-15;
    reg = H_norm2 < 1 ? 1e-7 : 1e-9;
  } else if (s.variant == 2) {
    return NQG_ERR_ARG;  // Tuned (four repeated solves) is not offered in batches
  }
  if (st.qp.precision == NQG_FP32) {  // FP32 factor: refinement always runs
    outer = std::max(outer, 2);
    inner = std::max(inner, 2);
  }
  if (inner > nqg::BATCH_MR_CAP) return NQG_ERR_SIZE;
  P.reg = reg;
  P.zero_thresh = reg;
  P.tol_abs = P.tol_rel = tol;
  P.outer = std::max(outer, 0);
  P.inner = std::max(inner, 0);
  P.eps_abs = s.eps_abs;
  P.max_iter_nas = s.max_iter_nas;
  return NQG_OK;
}

// Values of problem i into the host pool (original K values and the
// perturbed-diagonal flags).
void fill_values(nqg_batch *b, int i, std::vector<unsigned char> &pert_pool) {
  const HostQP &Q = b->qp[i];
  BProb &P = b->h_probs[i];
  nqg::Csc K;
  std::vector<double> kv;
  super_kkt(Q, K, &kv);
  std::copy(kv.begin(), kv.end(), b->h_dpool.begin() + P.o_kv);
  std::copy(Q.q.begin(), Q.q.end(), b->h_dpool.begin() + P.o_q);
  std::copy(Q.b.begin(), Q.b.end(), b->h_dpool.begin() + P.o_b);
  std::copy(Q.d.begin(), Q.d.end(), b->h_dpool.begin() + P.o_d);
  const int N = K.n;
  unsigned char *pf = pert_pool.data() + (P.o_pert - b->n_dbl * (int64_t)sizeof(double));
  for (int j = 0; j < N; ++j) pf[j] = std::abs(kv[K.p[j]]) < P.reg ? 1 : 0;
  double amax = 0.0;
  for (double v : kv) amax = std::max(amax, std::abs(v));
  P.reg32 = 3e-5 * (amax > 0 ? amax : 1.0);
}

// Queue resets and one persistent launch per tier, forked from the batch's
// stream and joined back into it.
int launch(nqg_batch *b) {
  if (cudaEventRecord(b->efork, b->stream) != cudaSuccess) return NQG_ERR_CUDA;
  for (size_t t = 0; t < b->tiers.size(); ++t) {
    TierLaunch &L = b->tiers[t];
    if (cudaStreamWaitEvent(L.stream, b->efork, 0) != cudaSuccess) return NQG_ERR_CUDA;
    if (cudaMemsetAsync(L.args.head, 0, sizeof(int), L.stream) != cudaSuccess) return NQG_ERR_CUDA;
    L.args.prof = b->args.prof;
    const int rc = b->set.qp.precision == NQG_FP32
                       ? nqg::launch_batch<float>(L.args, L.grid, b->threads, L.smem, L.stream)
                       : nqg::launch_batch<double>(L.args, L.grid, b->threads, L.smem, L.stream);
    if (rc) return rc;
    if (cudaEventRecord(L.done, L.stream) != cudaSuccess) return NQG_ERR_CUDA;
    if (cudaStreamWaitEvent(b->stream, L.done, 0) != cudaSuccess) return NQG_ERR_CUDA;
  }
  return NQG_OK;
}

}  // namespace

extern "C" void nqg_batch_default_settings(nqg_batch_settings *s) {
  if (!s) return;
  nqg_qp_default_settings(&s->qp);
  s->qp.eps_abs = 1e-8;
  s->refine = 0;
  s->refine_tol = 1e-12;
  s->threads = 0;
  s->use_graph = 1;
  s->stage = 0;
  s->share_factor = 1;
}

extern "C" int nqg_batch_create(const nqg_batch_settings *s, nqg_batch **out) {
  if (!out) return NQG_ERR_ARG;
  auto *b = new nqg_batch;
  if (s) b->set = *s;
  else nqg_batch_default_settings(&b->set);
  if ((b->set.qp.precision != NQG_FP64 && b->set.qp.precision != NQG_FP32) || b->set.qp.scaling != 0) {
    delete b;
    return NQG_ERR_ARG;
  }
  *out = b;
  return NQG_OK;
}

extern "C" int nqg_batch_add(nqg_batch *b, int n, const int *Hp, const int *Hi, const double *Hx, const double *q,
                             int meq, const int *Ap, const int *Ai, const double *Ax, const double *a, int mineq,
                             const int *Bp, const int *Bi, const double *Bx, const double *bineq) {
  if (!b || b->finalized) return NQG_ERR_STATE;
  if (n <= 0 || !Hp || !Hi || !Hx || !q || meq < 0 || mineq < 0) return NQG_ERR_ARG;
  if (meq > 0 && (!Ap || !Ai || !Ax || !a)) return NQG_ERR_ARG;
  if (mineq > 0 && (!Bp || !Bi || !Bx || !bineq)) return NQG_ERR_ARG;
  HostQP Q;
  Q.n = n;
  Q.meq = meq;
  Q.mineq = mineq;
  Q.Hp.assign(Hp, Hp + n + 1);
  Q.Hi.assign(Hi, Hi + Hp[n]);
  Q.Hx.assign(Hx, Hx + Hp[n]);
  Q.q.assign(q, q + n);
  for (int j = 0; j < n; ++j) {
    if (Hp[j + 1] < Hp[j]) return NQG_ERR_ARG;
    for (int k = Hp[j]; k < Hp[j + 1]; ++k)
      if (Hi[k] < j || Hi[k] >= n || (k > Hp[j] && Hi[k] <= Hi[k - 1])) return NQG_ERR_ARG;
  }
  auto take = [n](int m, const int *p, const int *ii, const double *x, std::vector<int> &P, std::vector<int> &I,
                  std::vector<double> &X) {
    P.assign(p, p + n + 1);
    I.assign(ii, ii + p[n]);
    X.assign(x, x + p[n]);
    for (int j = 0; j < n; ++j)
      for (int k = p[j]; k < p[j + 1]; ++k)
        if (ii[k] < 0 || ii[k] >= m || (k > p[j] && ii[k] <= ii[k - 1])) return false;
    return true;
  };
  if (meq > 0) {
    if (!take(meq, Ap, Ai, Ax, Q.Ap, Q.Ai, Q.Ax)) return NQG_ERR_ARG;
    Q.b.assign(a, a + meq);
  } else {
    Q.Ap.assign(n + 1, 0);
  }
  if (mineq > 0) {
    if (!take(mineq, Bp, Bi, Bx, Q.Cp, Q.Ci, Q.Cx)) return NQG_ERR_ARG;
    Q.d.assign(bineq, bineq + mineq);
  } else {
    Q.Cp.assign(n + 1, 0);
  }
  b->qp.push_back(std::move(Q));
  return (int)b->qp.size() - 1;
}

extern "C" int nqg_batch_finalize(nqg_batch *b) {
  if (!b || b->finalized) return NQG_ERR_STATE;
  const int np = (int)b->qp.size();
  if (np == 0) return NQG_ERR_ARG;
  // ---- patterns
  const int nrelax[3] = {4, 16, 48};
  const double zrelax[3] = {0.8, 0.1, 0.05};
  std::unordered_map<uint64_t, std::vector<int>> by_key;
  for (int i = 0; i < np; ++i) {
    HostQP &Q = b->qp[i];
    const uint64_t key = pattern_key(Q);
    int found = -1;
    for (int pidx : by_key[key])
      if (same_pattern(b->qp[b->pats[pidx].rep], Q)) found = pidx;
    if (found < 0) {
      HostPattern H;
      H.rep = i;
      std::string err = build_pattern(Q, H, nrelax, zrelax);
      if (!err.empty()) return fail(b, NQG_ERR_SYMBOLIC, err);
      found = (int)b->pats.size();
      b->pats.push_back(std::move(H));
      by_key[key].push_back(found);
    }
    Q.pat = found;
  }
  // ---- integer pool
  std::vector<int> ipool;
  std::vector<BPat> hp;
  int N_max = 0, nr_max = 1, w_max = 1, xs_max = 0, ss_max = 0, ns_max = 1, mi_max = 1, nlev_max = 1, nR_max = 1;
  for (HostPattern &H : b->pats) {
    BPat &P = H.P;
    auto put = [&ipool](const std::vector<int> &v) {
      const int o = (int)ipool.size();
      ipool.insert(ipool.end(), v.begin(), v.end());
      ipool.push_back(0);  // keeps every offset valid for empty arrays
      return o;
    };
    P.o_super = put(H.super);
    P.o_sparent = put(H.sparent);
    P.o_col2sup = put(H.col2sup);
    P.o_lpi = put(H.lpi);
    P.o_lpx = put(H.lpx);
    P.o_ls0 = put(H.ls0);
    P.o_perm0 = put(H.perm0);
    P.o_lvl_ptr = put(H.lvl_ptr);
    P.o_lvl_sn = put(H.lvl_sn);
    P.o_lev = put(H.lev);
    P.o_pair_ptr = put(H.pair_ptr);
    P.o_pair_mid = put(H.pair_mid);
    P.o_pair_d = put(H.pair_d);
    P.o_pair_lb = put(H.pair_lb);
    P.o_pair_ub = put(H.pair_ub);
    P.o_Rp = put(H.Rp);
    P.o_Rj = put(H.Rj);
    P.o_Rq = put(H.Rq);
    P.o_ent = put(H.ent);
    P.o_bt_ptr = put(H.bt_ptr);
    P.o_bt_var = put(H.bt_var);
    P.o_bt_q = put(H.bt_q);
    P.o_bt_rpos = put(H.bt_rpos);
    P.o_sn_con = put(H.sn_con);
    P.o_con_sn = put(H.con_sn);
    P.o_eq_ptr = put(H.eq_ptr);
    P.o_eq_var = put(H.eq_var);
    P.o_eq_q = put(H.eq_q);
    // records start on 16-byte boundaries (int4 loads)
    while (ipool.size() % 4) ipool.push_back(0);
    P.o_snrec = put(H.snrec);
    while (ipool.size() % 4) ipool.push_back(0);
    P.o_prec = put(H.prec);
    P.o_con_ptr = put(H.con_ptr);
    P.o_con_tgt = put(H.con_tgt);
    P.o_sn_big = put(H.sn_big);
    hp.push_back(P);
    N_max = std::max(N_max, P.N);
    nr_max = std::max(nr_max, P.max_nr);
    w_max = std::max(w_max, P.max_w);
    xs_max = std::max(xs_max, P.xsize);
    ss_max = std::max(ss_max, P.ssize);
    ns_max = std::max(ns_max, P.ns);
    mi_max = std::max(mi_max, P.mineq);
    nlev_max = std::max(nlev_max, P.nlev);
    nR_max = std::max(nR_max, P.nnzR);
  }
  if (ipool.size() > (size_t)INT32_MAX) return fail(b, NQG_ERR_SIZE, "integer work lists exceed 2^31 entries");
  // ---- per-problem settings and value layout
  b->h_probs.assign(np, BProb{});
  int64_t od = 0, oo = 0, oi = 0;
  int mr_max = 1;
  for (int i = 0; i < np; ++i) {
    const HostQP &Q = b->qp[i];
    const BPat &P = b->pats[Q.pat].P;
    BProb &R = b->h_probs[i];
    R.pat = Q.pat;
    int rc = problem_settings(b->set, Q, R);
    if (rc) return fail(b, rc, "unsupported settings (Tuned variant, or more than 10 refinement steps per restart)");
    mr_max = std::max(mr_max, R.inner);
    R.ws_n = -1;
    R.o_kv = od;
    od += P.nnzK;
    R.o_q = od;
    od += Q.n;
    R.o_b = od;
    od += Q.meq;
    R.o_d = od;
    od += Q.mineq;
    R.o_x = oo;
    oo += Q.n;
    R.o_y = oo;
    oo += Q.meq;
    R.o_z = oo;
    oo += Q.mineq;
    R.o_as = oi;
    oi += std::max(Q.mineq, 1);
  }
  b->n_dbl = od;
  int64_t pb = 0;
  for (int i = 0; i < np; ++i) {
    b->h_probs[i].o_pert = od * (int64_t)sizeof(double) + pb;
    pb += b->pats[b->qp[i].pat].P.N;
  }
  b->n_pert_bytes = pb;
  b->n_dout = oo;
  b->n_iout = oi;
  b->h_dpool.assign(od, 0.0);
  std::vector<unsigned char> pert(std::max<int64_t>(pb, 1), 0);
  for (int i = 0; i < np; ++i) fill_values(b, i, pert);
  // ---- groups of problems with identical matrices (pattern, K values,
  // perturbation flags, regularization): one shared cold factorization each
  std::vector<int> base_rep;
  for (int i = 0; i < np; ++i) b->h_probs[i].base = -1;
  if (b->set.share_factor) {
    auto kv_of = [&](int i) { return b->h_dpool.data() + b->h_probs[i].o_kv; };
    auto pf_of = [&](int i) { return pert.data() + (b->h_probs[i].o_pert - od * (int64_t)sizeof(double)); };
    std::unordered_map<uint64_t, std::vector<int>> cand;  // key -> representatives
    std::vector<int> members(np, 0), first_of(np, -1);
    for (int i = 0; i < np; ++i) {
      const BProb &R = b->h_probs[i];
      const BPat &Pp = b->pats[R.pat].P;
      uint64_t h = 1469598103934665603ull ^ (uint64_t)R.pat;
      const unsigned char *kb = reinterpret_cast<const unsigned char *>(kv_of(i));
      for (int64_t t = 0; t < (int64_t)Pp.nnzK * 8; ++t) h = (h ^ kb[t]) * 1099511628211ull;
      int rep = -1;
      for (int r : cand[h]) {
        const BProb &Q = b->h_probs[r];
        if (Q.pat == R.pat && Q.reg == R.reg && Q.reg32 == R.reg32 && Q.outer == R.outer && Q.inner == R.inner &&
            std::memcmp(kv_of(r), kv_of(i), (size_t)Pp.nnzK * sizeof(double)) == 0 &&
            std::memcmp(pf_of(r), pf_of(i), (size_t)Pp.N) == 0) {
          rep = r;
          break;
        }
      }
      if (rep < 0) {
        cand[h].push_back(i);
        rep = i;
      }
      first_of[i] = rep;
      members[rep]++;
    }
    std::vector<int> gid(np, -1);
    for (int i = 0; i < np; ++i) {
      const int rep = first_of[i];
      if (members[rep] < 2) continue;  // alone: nothing to share
      if (gid[rep] < 0) {
        gid[rep] = (int)base_rep.size();
        base_rep.push_back(rep);
      }
      b->h_probs[i].base = gid[rep];
    }
  }
  b->nbase = (int)base_rep.size();
  // ---- slot layout (one problem at a time per CTA)
  const size_t ts = b->set.qp.precision == NQG_FP32 ? sizeof(float) : sizeof(double);
  nqg::BSlot sl{};
  int64_t off = 0;
  auto seg = [&off](int64_t bytes) {
    const int64_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  sl.o_L = seg((int64_t)xs_max * ts);
  sl.o_D = seg((int64_t)2 * N_max * ts);
  sl.o_ls = seg((int64_t)ss_max * 4);
  sl.o_perm = seg((int64_t)N_max * 4);
  sl.o_iperm = seg((int64_t)N_max * 4);
  sl.o_lperm = seg((int64_t)N_max * 4);
  sl.o_mark = seg(ns_max);
  sl.o_piv = seg(ns_max);
  sl.o_alist = seg((int64_t)mi_max * 4);
  sl.o_vlist = seg((int64_t)ns_max * 4);
  sl.o_mlist = seg((int64_t)ns_max * 4);
  sl.o_Fv = seg((int64_t)nR_max * 8);
  sl.o_Rv = seg((int64_t)nR_max * 8);
  sl.o_cmask = seg((int64_t)ns_max * 8);
  sl.o_rhs = seg((int64_t)N_max * 8);
  sl.o_sol = seg((int64_t)N_max * 8);
  sl.o_r = seg((int64_t)N_max * 8);
  sl.o_w = seg((int64_t)N_max * 8);
  sl.o_tmp = seg((int64_t)N_max * 8);
  sl.o_V = seg((int64_t)(mr_max + 1) * N_max * 8);
  sl.o_Z = seg((int64_t)mr_max * N_max * ts);
  sl.bytes = off;
  // ---- launch shape: shared-memory tiers.  A problem whose factor and row
  // lists fit in a tier's staging space keeps them on chip while it runs;
  // each tier is one persistent launch (its queue, its slots), and the tiers
  // run side by side on forked streams.  Problems that fit no tier (or all
  // of them, with staging off) keep them in their slot (L2 / HBM).
  BQ_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  int dev = 0;
  BQ_CUDA(cudaGetDevice(&dev));
  BQ_CUDA(cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev));
  int smem_optin = 0;
  BQ_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  b->threads = b->set.threads > 0 ? b->set.threads : 128;
  if (b->threads % 32 || b->threads > 256) return fail(b, NQG_ERR_ARG, "threads must be a multiple of 32, at most 256");
  nqg::BArgs base_args{};
  base_args.N_max = N_max;
  base_args.w_max = w_max;
  base_args.nr_max = nr_max;
  base_args.ns_max = ns_max;
  base_args.mi_max = mi_max;
  base_args.nlev_max = nlev_max;
  base_args.stage_bytes = 0;
  const size_t static_smem = 8 * 1024;  // the kernel's own __shared__ variables, rounded up
  // Level-parallel factorization (a warp per supernode of at most 32 x 32)
  // for FP32 factors where its per-warp scratch keeps as many CTAs per SM as
  // the layout without it (FP64 factors measured faster on the CTA path);
  // NASOQ_GB300_BATCH_WARP_FACTOR=0 / 1 turns it off / on.
  {
    const char *e = std::getenv("NASOQ_GB300_BATCH_WARP_FACTOR");
    base_args.warp_factor = 0;
    if (e && std::string(e) == "1") {
      base_args.warp_factor = 1;
    } else if (!(e && std::string(e) == "0") && b->set.qp.precision == NQG_FP32) {
      nqg::BArgs with = base_args;
      with.warp_factor = 1;
      const size_t s0 = nqg::batch_smem_bytes(base_args, ts), s1 = nqg::batch_smem_bytes(with, ts);
      auto occ = [&](size_t sm, int *bps) {
        return b->set.qp.precision == NQG_FP32 ? nqg::batch_prepare<float>(b->threads, sm, sm, bps)
                                               : nqg::batch_prepare<double>(b->threads, sm, sm, bps);
      };
      int b0 = 0, b1 = 0;
      if ((int64_t)s1 + (int64_t)static_smem <= smem_optin && occ(s0, &b0) == NQG_OK && occ(s1, &b1) == NQG_OK &&
          b1 > 0 && b1 >= b0)
        base_args.warp_factor = 1;
    }
  }
  const size_t base_smem = nqg::batch_smem_bytes(base_args, ts);
  if ((int64_t)base_smem + (int64_t)static_smem > smem_optin)
    return fail(b, NQG_ERR_SIZE, "largest pattern exceeds the batched solver's shared memory");
  const int64_t stage_max = smem_optin - (int64_t)base_smem - (int64_t)static_smem;
  std::vector<int64_t> need(np);
  for (int i = 0; i < np; ++i) {
    const BPat &P = b->pats[b->qp[i].pat].P;
    need[i] = ((int64_t)P.xsize * (int64_t)ts + 15) / 16 * 16 + (int64_t)P.ssize * 4;
  }
  std::vector<int64_t> budgets;
  if (b->set.stage) {
    for (int64_t kb : {16, 32, 48, 64, 96, 128, 160, 192, 224})
      if (kb * 1024 <= stage_max) budgets.push_back(kb * 1024);
    if (budgets.empty() || budgets.back() < stage_max) budgets.push_back(stage_max / 16 * 16);
  }
  std::vector<int> tier_of(np, -1);  // index into budgets, -1: slot memory
  for (int i = 0; i < np; ++i)
    for (size_t t = 0; t < budgets.size(); ++t)
      if (need[i] <= budgets[t]) {
        tier_of[i] = (int)t;
        break;
      }
  // queue order inside every tier: largest problems first (longest-processing-time order)
  std::vector<int> order(np);
  for (int i = 0; i < np; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    if (tier_of[x] != tier_of[y]) return tier_of[x] == -1 ? true : (tier_of[y] == -1 ? false : tier_of[x] > tier_of[y]);
    const BPat &A = b->pats[b->qp[x].pat].P, &B = b->pats[b->qp[y].pat].P;
    const double cx = (double)A.xsize * (A.mineq + 1), cy = (double)B.xsize * (B.mineq + 1);
    return cx > cy;
  });
  b->tiers.clear();
  for (int q = 0; q < np;) {
    const int t = tier_of[order[q]];
    int e = q;
    while (e < np && tier_of[order[e]] == t) ++e;
    TierLaunch L;
    L.args = base_args;
    L.args.stage_bytes = t < 0 ? 0 : (int)budgets[t];
    L.smem = base_smem + (size_t)L.args.stage_bytes;
    L.order_off = q;
    L.nprob = e - q;
    b->tiers.push_back(L);
    q = e;
  }
  size_t smem_top = 0;
  for (auto &L : b->tiers) smem_top = std::max(smem_top, L.smem);
  int64_t nslots = 0;
  for (auto &L : b->tiers) {
    int bps = 0;
    int rc = b->set.qp.precision == NQG_FP32 ? nqg::batch_prepare<float>(b->threads, smem_top, L.smem, &bps)
                                            : nqg::batch_prepare<double>(b->threads, smem_top, L.smem, &bps);
    if (rc || bps <= 0) return fail(b, NQG_ERR_CUDA, "no resident CTA fits the batched kernel");
    L.bps = bps;
    L.grid = std::min(L.nprob, bps * b->num_sms);
    L.slot_off = nslots;
    nslots += L.grid;
  }
  b->smem = smem_top;
  b->grid = (int)nslots;
  b->blocks_per_sm = b->tiers.empty() ? 0 : b->tiers.front().bps;
  // ---- device
  BQ_CUDA(cudaMalloc(&b->d_pats, hp.size() * sizeof(BPat)));
  BQ_CUDA(cudaMemcpy(b->d_pats, hp.data(), hp.size() * sizeof(BPat), cudaMemcpyHostToDevice));
  BQ_CUDA(cudaMalloc(&b->d_probs, np * sizeof(BProb)));
  BQ_CUDA(cudaMalloc(&b->d_ipool, ipool.size() * sizeof(int)));
  BQ_CUDA(cudaMemcpy(b->d_ipool, ipool.data(), ipool.size() * sizeof(int), cudaMemcpyHostToDevice));
  BQ_CUDA(cudaMalloc(&b->d_dpool, od * sizeof(double) + std::max<int64_t>(pb, 1)));
  BQ_CUDA(cudaMemcpy(b->d_dpool, b->h_dpool.data(), od * sizeof(double), cudaMemcpyHostToDevice));
  BQ_CUDA(cudaMemcpy(reinterpret_cast<unsigned char *>(b->d_dpool) + od * sizeof(double), pert.data(), pb,
                     cudaMemcpyHostToDevice));
  BQ_CUDA(cudaMalloc(&b->d_dout, std::max<int64_t>(oo, 1) * sizeof(double)));
  BQ_CUDA(cudaMemset(b->d_dout, 0, std::max<int64_t>(oo, 1) * sizeof(double)));
  BQ_CUDA(cudaMalloc(&b->d_iout, std::max<int64_t>(oi, 1) * sizeof(int)));
  BQ_CUDA(cudaMalloc(&b->d_res, np * sizeof(BResult)));
  BQ_CUDA(cudaMalloc(&b->d_order, np * sizeof(int)));
  BQ_CUDA(cudaMemcpy(b->d_order, order.data(), np * sizeof(int), cudaMemcpyHostToDevice));
  BQ_CUDA(cudaMalloc(&b->d_head, std::max<size_t>(b->tiers.size(), 1) * sizeof(int)));
  BQ_CUDA(cudaMalloc(&b->d_slots, (size_t)std::max<int64_t>(nslots, 1) * sl.bytes));
  if (b->nbase > 0) {
    BQ_CUDA(cudaMalloc(&b->d_bases, (size_t)b->nbase * sl.bytes));
    BQ_CUDA(cudaMalloc(&b->d_base_rep, (size_t)b->nbase * sizeof(int)));
    BQ_CUDA(cudaMemcpy(b->d_base_rep, base_rep.data(), (size_t)b->nbase * sizeof(int), cudaMemcpyHostToDevice));
  }
  BQ_CUDA(cudaMemcpy(b->d_probs, b->h_probs.data(), np * sizeof(BProb), cudaMemcpyHostToDevice));
  BQ_CUDA(cudaEventCreateWithFlags(&b->e0, cudaEventDefault));
  BQ_CUDA(cudaEventCreateWithFlags(&b->e1, cudaEventDefault));
  BQ_CUDA(cudaEventCreateWithFlags(&b->efork, cudaEventDisableTiming));
  for (size_t t = 0; t < b->tiers.size(); ++t) {
    TierLaunch &L = b->tiers[t];
    BQ_CUDA(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
    BQ_CUDA(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming));
    nqg::BArgs &A = L.args;
    A.pats = b->d_pats;
    A.probs = b->d_probs;
    A.ipool = b->d_ipool;
    A.dpool = b->d_dpool;
    A.dout = b->d_dout;
    A.iout = b->d_iout;
    A.res = b->d_res;
    A.order = b->d_order + L.order_off;
    A.head = b->d_head + t;
    A.nprob = L.nprob;
    A.slots = b->d_slots + (size_t)L.slot_off * sl.bytes;
    A.slot = sl;
    A.refine = b->set.refine;
    A.refine_tol = b->set.refine_tol;
    A.mr_max = mr_max;
    A.prof = nullptr;
    A.bases = b->d_bases;
    A.base_rep = b->d_base_rep;
    A.nbase = b->nbase;
    A.mode = 0;
  }
  b->args.slot = sl;
  // ---- the groups' shared factorizations (once: the matrices never change)
  if (b->nbase > 0) {
    TierLaunch &T0 = b->tiers.front();
    nqg::BArgs A = T0.args;
    A.mode = 1;
    A.stage_bytes = 0;
    A.slots = b->d_slots;
    A.head = b->d_head;
    BQ_CUDA(cudaMemsetAsync(A.head, 0, sizeof(int), b->stream));
    const int grid = std::min(b->nbase, T0.bps * b->num_sms);
    const size_t smem = base_smem;
    const int rc = b->set.qp.precision == NQG_FP32 ? nqg::launch_batch<float>(A, grid, b->threads, smem, b->stream)
                                                   : nqg::launch_batch<double>(A, grid, b->threads, smem, b->stream);
    if (rc) return fail(b, rc, "launch of the shared factorizations failed");
    BQ_CUDA(cudaStreamSynchronize(b->stream));
  }
  b->finalized = true;
  return NQG_OK;
}

// New q / b / d for every problem, concatenated in problem order (any may be
// NULL: unchanged).  One copy per given vector into a staging buffer, then
// one kernel scatters every problem's segment into the value pool, both on
// the batch's stream; `sync` waits for them and keeps the host copies of the
// vectors current (nothing reads those after finalize).
static int set_vectors_impl(nqg_batch *b, const double *q_all, const double *beq_all, const double *d_all,
                            bool sync) {
  if (!b || !b->finalized) return NQG_ERR_STATE;
  const int np = (int)b->qp.size();
  int64_t tq = 0, tb = 0, td = 0;
  for (const HostQP &Q : b->qp) {
    tq += Q.n;
    tb += Q.meq;
    td += Q.mineq;
  }
  if (!b->d_vstage) {
    b->n_vstage = tq + tb + td;
    BQ_CUDA(cudaMalloc(&b->d_vstage, std::max<int64_t>(b->n_vstage, 1) * sizeof(double)));
    BQ_CUDA(cudaMalloc(&b->d_voff, (size_t)np * 3 * sizeof(int64_t)));
  }
  // segment offsets of every problem (-1: vector not given), kept in the
  // batch so that an asynchronous copy of them never reads freed memory
  std::vector<int64_t> &off = b->h_voff;
  off.assign((size_t)np * 3, -1);
  int64_t oq = 0, ob = tq, odd = tq + tb;
  for (int i = 0; i < np; ++i) {
    HostQP &Q = b->qp[i];
    if (q_all) {
      if (sync) std::copy(q_all + oq, q_all + oq + Q.n, Q.q.begin());
      off[3 * i] = oq;
    }
    if (beq_all) {
      if (sync) std::copy(beq_all + (ob - tq), beq_all + (ob - tq) + Q.meq, Q.b.begin());
      off[3 * i + 1] = ob;
    }
    if (d_all) {
      if (sync) std::copy(d_all + (odd - tq - tb), d_all + (odd - tq - tb) + Q.mineq, Q.d.begin());
      off[3 * i + 2] = odd;
    }
    oq += Q.n;
    ob += Q.meq;
    odd += Q.mineq;
  }
  if (q_all && tq)
    BQ_CUDA(cudaMemcpyAsync(b->d_vstage, q_all, tq * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  if (beq_all && tb)
    BQ_CUDA(cudaMemcpyAsync(b->d_vstage + tq, beq_all, tb * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  if (d_all && td)
    BQ_CUDA(cudaMemcpyAsync(b->d_vstage + tq + tb, d_all, td * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  BQ_CUDA(cudaMemcpyAsync(b->d_voff, off.data(), off.size() * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
  const int rc = nqg::batch_scatter_vectors(np, b->d_probs, b->d_pats, b->d_voff, b->d_vstage, b->d_dpool, b->stream);
  if (rc) return fail(b, rc, "vector scatter failed");
  if (sync) BQ_CUDA(cudaStreamSynchronize(b->stream));
  return NQG_OK;
}

extern "C" int nqg_batch_set_vectors(nqg_batch *b, const double *q_all, const double *beq_all,
                                     const double *d_all) {
  return set_vectors_impl(b, q_all, beq_all, d_all, true);
}

extern "C" int nqg_batch_set_vectors_async(nqg_batch *b, const double *q_all, const double *beq_all,
                                           const double *d_all) {
  return set_vectors_impl(b, q_all, beq_all, d_all, false);
}

extern "C" int nqg_batch_set_warm_start(nqg_batch *b, int i, int n_as, const int *as) {
  // Proposed active set of problem i for the next solve (n_as < 0: cold start).
  if (!b || !b->finalized) return NQG_ERR_STATE;
  if (i < 0 || i >= (int)b->qp.size()) return NQG_ERR_ARG;
  HostQP &Q = b->qp[i];
  BProb &P = b->h_probs[i];
  if (n_as < 0) {
    P.ws_n = -1;
  } else {
    if (n_as > Q.mineq || (n_as > 0 && !as)) return NQG_ERR_ARG;
    for (int t = 0; t < n_as; ++t)
      if (as[t] < 0 || as[t] >= Q.mineq) return NQG_ERR_ARG;
    P.ws_n = n_as;
    if (n_as > 0)
      BQ_CUDA(cudaMemcpyAsync(b->d_iout + P.o_as, as, n_as * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  }
  BQ_CUDA(cudaMemcpyAsync(b->d_probs + i, &P, sizeof(BProb), cudaMemcpyHostToDevice, b->stream));
  BQ_CUDA(cudaStreamSynchronize(b->stream));
  return NQG_OK;
}

extern "C" int nqg_batch_warm_start_from_scores(nqg_batch *b, const float *d_scores, int ld, float threshold) {
  // Warm-start sets of every problem from device-resident scores (row i:
  // problem i's constraints); see k_ws_scores.  Runs on the batch's stream.
  if (!b || !b->finalized) return NQG_ERR_STATE;
  if (!d_scores || ld <= 0) return NQG_ERR_ARG;
  const int np = (int)b->qp.size();
  int rc = nqg::batch_ws_from_scores(np, b->d_probs, b->d_pats, b->d_ipool, b->d_dpool, b->d_iout, d_scores, ld,
                                     threshold, b->stream);
  if (rc) return fail(b, rc, "warm-start kernel launch failed");
  for (auto &P : b->h_probs) P.ws_n = 0;  // device copies now hold the sets
  return NQG_OK;
}

extern "C" int nqg_batch_clear_warm_starts(nqg_batch *b) {
  // Every problem back to a cold start.
  if (!b || !b->finalized) return NQG_ERR_STATE;
  const int np = (int)b->qp.size();
  int rc = nqg::batch_ws_clear(np, b->d_probs, b->stream);
  if (rc) return fail(b, rc, "warm-start kernel launch failed");
  for (auto &P : b->h_probs) P.ws_n = -1;
  BQ_CUDA(cudaStreamSynchronize(b->stream));
  return NQG_OK;
}

extern "C" int nqg_batch_solve_async(nqg_batch *b) {
  // Enqueues one solve of every problem on the batch's stream (captured once
  // into a CUDA graph of the queue reset and the persistent kernel).
  if (!b || !b->finalized) return NQG_ERR_STATE;
  if (b->set.use_graph) {
    if (!b->gexec) {
      BQ_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      int rc = launch(b);
      cudaGraph_t g = nullptr;
      cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
      if (rc || ec != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(b, NQG_ERR_CUDA, "graph capture of the batched solve failed");
      }
      b->graph = g;
      BQ_CUDA(cudaGraphInstantiate(&b->gexec, g, 0));
    }
    BQ_CUDA(cudaGraphLaunch(b->gexec, b->stream));
  } else {
    int rc = launch(b);
    if (rc) return fail(b, rc, "launch of the batched kernel failed");
  }
  return NQG_OK;
}

extern "C" int nqg_batch_solve(nqg_batch *b) {
  if (!b || !b->finalized) return NQG_ERR_STATE;
  BQ_CUDA(cudaEventRecord(b->e0, b->stream));
  int rc = nqg_batch_solve_async(b);
  if (rc) return rc;
  BQ_CUDA(cudaEventRecord(b->e1, b->stream));
  BQ_CUDA(cudaStreamSynchronize(b->stream));
  float ms = 0.f;
  BQ_CUDA(cudaEventElapsedTime(&ms, b->e0, b->e1));
  b->last_ms = ms;
  return NQG_OK;
}

extern "C" int nqg_batch_get(nqg_batch *b, int i, double *x, double *y, double *z, int *active_set,
                             nqg_qp_result *res) {
  if (!b || !b->finalized) return NQG_ERR_STATE;
  if (i < 0 || i >= (int)b->qp.size()) return NQG_ERR_ARG;
  const HostQP &Q = b->qp[i];
  const BProb &P = b->h_probs[i];
  BResult R{};
  BQ_CUDA(cudaMemcpy(&R, b->d_res + i, sizeof(BResult), cudaMemcpyDeviceToHost));
  if (x) BQ_CUDA(cudaMemcpy(x, b->d_dout + P.o_x, Q.n * sizeof(double), cudaMemcpyDeviceToHost));
  if (y && Q.meq) BQ_CUDA(cudaMemcpy(y, b->d_dout + P.o_y, Q.meq * sizeof(double), cudaMemcpyDeviceToHost));
  if (z && Q.mineq) BQ_CUDA(cudaMemcpy(z, b->d_dout + P.o_z, Q.mineq * sizeof(double), cudaMemcpyDeviceToHost));
  if (active_set && Q.mineq)
    BQ_CUDA(cudaMemcpy(active_set, b->d_iout + P.o_as, Q.mineq * sizeof(int), cudaMemcpyDeviceToHost));
  if (res) {
    res->status = R.status;
    res->num_iter = R.num_iter;
    res->active_size = R.active_size;
    res->objective = R.objective;
    res->primal_obj = R.primal_obj;
    res->dual_obj = R.dual_obj;
    res->lag_res = R.lag_res;
    res->cons_sat_norm = R.cons_sat_norm;
    res->non_negativity_infn = R.non_negativity_infn;
    res->complementarity_infn = R.complementarity_infn;
    res->total_seconds = b->last_ms * 1e-3;
    res->factor_seconds = 0.0;
  }
  return R.flags & nqg::ST_NONFINITE ? NQG_WARN_NONFINITE : (R.flags & nqg::ST_ZERO_PIVOT ? NQG_WARN_ZERO_PIVOT : NQG_OK);
}

extern "C" int nqg_batch_get_all(nqg_batch *b, double *x_all, double *y_all, double *z_all, nqg_batch_stats *stats) {
  // Every problem's x / y / z, concatenated in problem order (any may be NULL),
  // and per-problem statistics (nprob entries).
  if (!b || !b->finalized) return NQG_ERR_STATE;
  const int np = (int)b->qp.size();
  std::vector<double> out;
  if (x_all || y_all || z_all) {
    out.resize(std::max<int64_t>(b->n_dout, 1));
    BQ_CUDA(cudaMemcpyAsync(out.data(), b->d_dout, b->n_dout * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  }
  std::vector<BResult> R(np);
  BQ_CUDA(cudaMemcpyAsync(R.data(), b->d_res, np * sizeof(BResult), cudaMemcpyDeviceToHost, b->stream));
  BQ_CUDA(cudaStreamSynchronize(b->stream));
  int64_t ox = 0, oy = 0, oz = 0;
  for (int i = 0; i < np; ++i) {
    const HostQP &Q = b->qp[i];
    const BProb &P = b->h_probs[i];
    if (x_all) std::copy(out.begin() + P.o_x, out.begin() + P.o_x + Q.n, x_all + ox);
    if (y_all) std::copy(out.begin() + P.o_y, out.begin() + P.o_y + Q.meq, y_all + oy);
    if (z_all) std::copy(out.begin() + P.o_z, out.begin() + P.o_z + Q.mineq, z_all + oz);
    ox += Q.n;
    oy += Q.meq;
    oz += Q.mineq;
    if (stats) {
      nqg_batch_stats &s = stats[i];
      s.status = R[i].status;
      s.num_iter = R[i].num_iter;
      s.active_size = R[i].active_size;
      s.flags = R[i].flags;
      s.refine_steps = R[i].refine_steps;
      s.solves = R[i].solves;
      s.warm_dropped = R[i].warm_dropped;
      s.objective = R[i].objective;
      s.lag_res = R[i].lag_res;
      s.cons_sat_norm = R[i].cons_sat_norm;
      s.non_negativity_infn = R[i].non_negativity_infn;
      s.complementarity_infn = R[i].complementarity_infn;
    }
  }
  return NQG_OK;
}

extern "C" int nqg_batch_get_info(const nqg_batch *b, nqg_batch_info *info) {
  if (!b || !info) return NQG_ERR_ARG;
  info->nprob = (int)b->qp.size();
  info->npatterns = (int)b->pats.size();
  info->grid = b->grid;
  info->threads = b->threads;
  info->blocks_per_sm = b->blocks_per_sm;
  info->warp_factor = b->tiers.empty() ? 0 : b->tiers.front().args.warp_factor;
  info->smem_bytes = (int64_t)b->smem;
  info->slot_bytes = b->args.slot.bytes;
  info->last_ms = b->last_ms;
  return NQG_OK;
}

extern "C" int nqg_batch_set_profiling(nqg_batch *b, int on) {
  // Per-phase cycle counters of the next solves (summed over problems); a
  // change rebuilds the CUDA graph.
  if (!b || !b->finalized) return NQG_ERR_STATE;
  if (on && !b->d_prof) {
    BQ_CUDA(cudaMalloc(&b->d_prof, nqg::BATCH_PROFILE_COUNTERS * sizeof(unsigned long long)));
    BQ_CUDA(cudaMemset(b->d_prof, 0, nqg::BATCH_PROFILE_COUNTERS * sizeof(unsigned long long)));
  }
  b->args.prof = on ? b->d_prof : nullptr;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->gexec = nullptr;
  b->graph = nullptr;
  return NQG_OK;
}

extern "C" int nqg_batch_get_profile(nqg_batch *b, unsigned long long *counters, int n) {
  // Copies (and resets) the per-phase counters (see include/nasoq_gb300.h).
  if (!b || !b->finalized || !counters || n <= 0) return NQG_ERR_ARG;
  if (!b->d_prof) {
    for (int k = 0; k < n; ++k) counters[k] = 0;
    return NQG_OK;
  }
  unsigned long long h[nqg::BATCH_PROFILE_COUNTERS] = {};
  BQ_CUDA(cudaMemcpy(h, b->d_prof, sizeof h, cudaMemcpyDeviceToHost));
  BQ_CUDA(cudaMemset(b->d_prof, 0, sizeof h));
  for (int k = 0; k < n && k < nqg::BATCH_PROFILE_COUNTERS; ++k) counters[k] = h[k];
  return NQG_OK;
}

extern "C" int nqg_batch_get_stream(const nqg_batch *b, void **stream) {
  if (!b || !stream || !b->finalized) return NQG_ERR_ARG;
  *stream = b->stream;
  return NQG_OK;
}

extern "C" const char *nqg_batch_last_error(const nqg_batch *b) { return b ? b->last_error.c_str() : ""; }

extern "C" int nqg_batch_destroy(nqg_batch *b) {
  if (!b) return NQG_ERR_ARG;
  if (b->stream) cudaStreamSynchronize(b->stream);
  free_device(b);
  for (auto &L : b->tiers) {
    if (L.stream) cudaStreamDestroy(L.stream);
    if (L.done) cudaEventDestroy(L.done);
  }
  if (b->efork) cudaEventDestroy(b->efork);
  if (b->e0) cudaEventDestroy(b->e0);
  if (b->e1) cudaEventDestroy(b->e1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return NQG_OK;
}
