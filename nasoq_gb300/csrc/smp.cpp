// Reader of the SMP QP file format (reference smp-format/smp_format.h:174-233,
// SMP::load) and its conversion to the solver's form
//     min 1/2 x'Hx + q'x   s.t.   A x = b,  C x <= d
// (reference QPFormatConverter::smp_to_ie, smp-format/mp_format_converter.h:
// 681-712, with the bounds-to-rows rule of find_inequalities_by_bounds,
// :264-433).
//
// An SMP file is a list of YAML block scalars ("Key": |) whose indented
// bodies are MatrixMarket texts: "Quadratic" (H, symmetric, lower triangle),
// "Linear" (q), "Equality" (A), "Equality bounds" (b), "Inequality" (C),
// "Inequality l-bounds" / "Inequality u-bounds" (l <= C x <= u), "Fixed"
// (constant objective term), "Primals", "Duals", "Optimal objective" and
// "Description".  Keys are matched case-insensitively after trimming; an
// unknown key, or a key given twice, makes the file invalid (as for the
// reference loader).  A bound of magnitude 1e20 stands for infinity.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "nasoq_gb300.h"

namespace {

constexpr double kInf = 1e20;  // the format's infinity

struct Sparse {
  int m = 0, n = 0;
  std::vector<int> p, i;
  std::vector<double> x;
  bool present = false;
};

struct DenseV {
  std::vector<double> v;
  bool present = false;
};

std::string lower_trim(std::string s) {
  for (char &c : s) c = (char)std::tolower((unsigned char)c);
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// Reads the next whitespace-separated token of the stream.
bool token(std::istream &in, std::string &t) { return static_cast<bool>(in >> t); }

bool number(std::istream &in, double &v) {
  std::string t;
  if (!token(in, t)) return false;
  char *end = nullptr;
  v = std::strtod(t.c_str(), &end);
  return end && *end == '\0';
}

// The MatrixMarket banner and size line of one block.
struct MtxHeader {
  bool coordinate = true, symmetric = false;
  int m = 0, n = 0;
  int64_t nnz = 0;
};

bool read_mtx_header(std::istream &in, MtxHeader &h, std::string &err) {
  std::string line;
  do {
    if (!std::getline(in, line)) {
      err = "MatrixMarket header missing";
      return false;
    }
    line = lower_trim(line);
  } while (line.empty());
  std::istringstream bs(line);
  std::string banner, obj, fmt, field, shape;
  if (!(bs >> banner >> obj >> fmt >> field >> shape) || banner != "%%matrixmarket" || obj != "matrix") {
    err = "invalid MatrixMarket banner: " + line;
    return false;
  }
  if (fmt == "coordinate") h.coordinate = true;
  else if (fmt == "array") h.coordinate = false;
  else {
    err = "unsupported MatrixMarket format: " + fmt;
    return false;
  }
  if (field != "real") {
    err = "only real MatrixMarket values are read: " + field;
    return false;
  }
  if (shape == "symmetric") h.symmetric = true;
  else if (shape != "general") {
    err = "unsupported MatrixMarket shape: " + shape;
    return false;
  }
  // comment lines, then the sizes
  do {
    if (!std::getline(in, line)) {
      err = "MatrixMarket sizes missing";
      return false;
    }
    line = lower_trim(line);
  } while (line.empty() || line[0] == '%');
  std::istringstream ss(line);
  if (h.coordinate) {
    if (!(ss >> h.m >> h.n >> h.nnz)) {
      err = "MatrixMarket sizes missing";
      return false;
    }
  } else {
    if (!(ss >> h.m >> h.n)) {
      err = "MatrixMarket sizes missing";
      return false;
    }
    h.nnz = (int64_t)h.m * h.n;
  }
  return h.m >= 0 && h.n >= 0 && h.nnz >= 0;
}

// Coordinate block -> CSC with rows sorted in every column.  insert_diag: an
// empty column gets an explicit zero diagonal (the Hessian block).
bool read_sparse(std::istream &in, Sparse &S, bool insert_diag, std::string &err) {
  MtxHeader h;
  if (!read_mtx_header(in, h, err)) return false;
  if (!h.coordinate) {
    err = "a matrix block must be in coordinate format";
    return false;
  }
  struct T {
    int r, c;
    double v;
  };
  std::vector<T> t((size_t)h.nnz);
  for (auto &e : t) {
    double r, c;
    if (!number(in, r) || !number(in, c) || !number(in, e.v)) {
      err = "truncated MatrixMarket entries";
      return false;
    }
    e.r = (int)r - 1;
    e.c = (int)c - 1;
    if (e.r < 0 || e.r >= h.m || e.c < 0 || e.c >= h.n) {
      err = "MatrixMarket entry out of range";
      return false;
    }
  }
  std::stable_sort(t.begin(), t.end(), [](const T &a, const T &b) { return a.c < b.c || (a.c == b.c && a.r < b.r); });
  S.m = h.m;
  S.n = h.n;
  S.p.assign(h.n + 1, 0);
  S.i.clear();
  S.x.clear();
  size_t k = 0;
  for (int j = 0; j < h.n; ++j) {
    const size_t k0 = k;
    while (k < t.size() && t[k].c == j) {
      S.i.push_back(t[k].r);
      S.x.push_back(t[k].v);
      ++k;
    }
    if (k == k0 && insert_diag) {
      S.i.push_back(j);
      S.x.push_back(0.0);
    }
    S.p[j + 1] = (int)S.i.size();
  }
  S.present = true;
  return true;
}

bool read_dense(std::istream &in, DenseV &D, std::string &err) {
  MtxHeader h;
  if (!read_mtx_header(in, h, err)) return false;
  if (h.coordinate) {
    err = "a vector block must be in array format";
    return false;
  }
  D.v.resize((size_t)h.nnz);
  for (double &v : D.v)
    if (!number(in, v)) {
      err = "truncated MatrixMarket array";
      return false;
    }
  D.present = true;
  return true;
}

bool near(double a, double b) { return !std::isnan(a) && !std::isnan(b) && !(std::abs(a - b) > 1e-6); }

}  // namespace

struct nqg_qp_data {
  int n = 0;
  Sparse H, A, C;   // C after the bounds-to-rows conversion
  DenseV q, b, d, l, u, primals, duals;
  double fixed = 0.0, optimal_obj = 0.0;
  std::string description, error;
};

namespace {

int smp_parse(std::istream &in, nqg_qp_data &Q) {
  std::string line;
  Sparse Craw;
  while (std::getline(in, line)) {
    const std::string key = lower_trim(line);
    if (key.empty()) continue;
    bool ok = true;
    auto once = [&](bool present) {
      if (present) Q.error = "key given twice: " + key;
      return !present;
    };
    if (key == "\"quadratic\": |") ok = once(Q.H.present) && read_sparse(in, Q.H, true, Q.error);
    else if (key == "\"linear\": |") ok = once(Q.q.present) && read_dense(in, Q.q, Q.error);
    else if (key == "\"equality\": |") ok = once(Q.A.present) && read_sparse(in, Q.A, false, Q.error);
    else if (key == "\"equality bounds\": |") ok = once(Q.b.present) && read_dense(in, Q.b, Q.error);
    else if (key == "\"inequality\": |") ok = once(Craw.present) && read_sparse(in, Craw, false, Q.error);
    else if (key == "\"inequality l-bounds\": |") ok = once(Q.l.present) && read_dense(in, Q.l, Q.error);
    else if (key == "\"inequality u-bounds\": |") ok = once(Q.u.present) && read_dense(in, Q.u, Q.error);
    else if (key == "\"primals\": |") ok = once(Q.primals.present) && read_dense(in, Q.primals, Q.error);
    else if (key == "\"duals\": |") ok = once(Q.duals.present) && read_dense(in, Q.duals, Q.error);
    else if (key == "\"fixed\": |") ok = number(in, Q.fixed);
    else if (key == "\"optimal objective\": |") ok = number(in, Q.optimal_obj);
    else if (key == "\"description\": |" || key == "\"description\":") {
      // indented lines that follow
      std::streampos pos = in.tellg();
      while (std::getline(in, line)) {
        if (line.compare(0, 2, "  ") != 0) {
          if (!line.empty() && line[0] == '-') {
            pos = in.tellg();
            continue;
          }
          in.clear();
          in.seekg(pos);
          break;
        }
        const size_t a = line.find_first_not_of(" \t");
        Q.description += (a == std::string::npos ? std::string() : line.substr(a)) + "\n";
        pos = in.tellg();
      }
    } else if (key.find(':') != std::string::npos) {
      Q.error = "unknown key: " + key;
      return NQG_ERR_ARG;
    }
    if (!ok) {
      if (Q.error.empty()) Q.error = "malformed block after " + key;
      return NQG_ERR_ARG;
    }
  }
  // number of variables: the first block that fixes it
  Q.n = Q.H.present ? Q.H.n : 0;
  if (!Q.n && Q.q.present) Q.n = (int)Q.q.v.size();
  if (!Q.n && Q.A.present) Q.n = Q.A.n;
  if (!Q.n && Craw.present) Q.n = Craw.n;
  if (!Q.n && Q.primals.present) Q.n = (int)Q.primals.v.size();
  const int n = Q.n;
  if (!Q.H.present) {  // all-zero Hessian: explicit zero diagonal
    Q.H.m = Q.H.n = n;
    Q.H.p.resize(n + 1);
    for (int j = 0; j <= n; ++j) Q.H.p[j] = j;
    Q.H.i.resize(n);
    for (int j = 0; j < n; ++j) Q.H.i[j] = j;
    Q.H.x.assign(n, 0.0);
  }
  if (!Q.q.present) Q.q.v.assign(n, 0.0);
  if ((int)Q.q.v.size() != n || Q.H.m != n || Q.H.n != n) {
    Q.error = "inconsistent Hessian / linear term sizes";
    return NQG_ERR_ARG;
  }
  if (!Q.A.present) {
    Q.A.m = 0;
    Q.A.n = n;
    Q.A.p.assign(n + 1, 0);
  }
  if (Q.A.n != n || (int)Q.b.v.size() != Q.A.m) {
    Q.error = "inconsistent equality block sizes";
    return NQG_ERR_ARG;
  }
  // inequalities: l <= C x <= u  ->  rows of C x <= d
  Q.C.n = n;
  Q.C.p.assign(n + 1, 0);
  if (!Craw.present || Craw.m == 0) {
    Q.C.m = 0;
    return NQG_OK;
  }
  if (Craw.n != n) {
    Q.error = "inconsistent inequality block size";
    return NQG_ERR_ARG;
  }
  const int mc = Craw.m;
  std::vector<double> l(mc, -kInf), u(mc, kInf);
  if (Q.u.present) {
    if ((int)Q.u.v.size() != mc) {
      Q.error = "inconsistent inequality bound sizes";
      return NQG_ERR_ARG;
    }
    u = Q.u.v;
  }
  if (!Q.l.present) {
    // no lower bounds: C and u as given (reference smp_to_ie, :695-698)
    Q.C = Craw;
    Q.d.v = u;
    Q.d.present = true;
    return NQG_OK;
  }
  if ((int)Q.l.v.size() != mc) {
    Q.error = "inconsistent inequality bound sizes";
    return NQG_ERR_ARG;
  }
  l = Q.l.v;
  // rows of C (its transpose, column k = row k)
  std::vector<int> rp(mc + 1, 0), ri(Craw.i.size());
  std::vector<double> rx(Craw.i.size());
  for (int r : Craw.i) rp[r + 1]++;
  for (int r = 0; r < mc; ++r) rp[r + 1] += rp[r];
  {
    std::vector<int> pos(rp.begin(), rp.end() - 1);
    for (int j = 0; j < n; ++j)
      for (int q = Craw.p[j]; q < Craw.p[j + 1]; ++q) {
        const int t = pos[Craw.i[q]]++;
        ri[t] = j;
        rx[t] = Craw.x[q];
      }
  }
  // each row becomes 0, 1 or 2 rows of C x <= d, in order: u first (+row),
  // then -l (-row)
  struct Out {
    int row;
    double sign, rhs;
  };
  std::vector<Out> rows;
  for (int k = 0; k < mc; ++k) {
    const double lk = std::abs(l[k]) < 1e-14 ? 0.0 : l[k];
    const double uk = std::abs(u[k]) < 1e-14 ? 0.0 : u[k];
    if ((near(lk, -kInf) && near(uk, kInf)) || (near(lk, kInf) && near(uk, kInf)) ||
        (near(lk, -kInf) && near(uk, -kInf)))
      continue;  // no constraint
    if (near(lk, uk)) {
      Q.error = "an inequality row with equal bounds (give it as an equality)";
      return NQG_ERR_ARG;
    }
    if (near(lk, -kInf)) {
      rows.push_back({k, 1.0, uk});
    } else if (near(uk, kInf)) {
      rows.push_back({k, -1.0, -lk});
    } else {
      rows.push_back({k, 1.0, uk});
      rows.push_back({k, -1.0, -lk});
    }
  }
  const int mo = (int)rows.size();
  Q.C.m = mo;
  Q.d.v.resize(mo);
  Q.d.present = true;
  // C (column-wise) from the output rows
  std::vector<int> cnt(n, 0);
  for (const Out &o : rows)
    for (int t = rp[o.row]; t < rp[o.row + 1]; ++t) cnt[ri[t]]++;
  for (int j = 0; j < n; ++j) Q.C.p[j + 1] = Q.C.p[j] + cnt[j];
  Q.C.i.resize(Q.C.p[n]);
  Q.C.x.resize(Q.C.p[n]);
  std::vector<int> pos(Q.C.p.begin(), Q.C.p.end() - 1);
  for (int k = 0; k < mo; ++k) {
    const Out &o = rows[k];
    Q.d.v[k] = o.rhs;
    for (int t = rp[o.row]; t < rp[o.row + 1]; ++t) {
      const int w = pos[ri[t]]++;
      Q.C.i[w] = k;
      Q.C.x[w] = o.sign * rx[t];
    }
  }
  Q.C.present = true;
  return NQG_OK;
}

}  // namespace

extern "C" int nqg_smp_load(const char *path, nqg_qp_data **out) {
  if (!path || !out) return NQG_ERR_ARG;
  *out = nullptr;
  std::ifstream in(path);
  if (!in.is_open()) return NQG_ERR_ARG;
  auto *Q = new nqg_qp_data;
  const int rc = smp_parse(in, *Q);
  *out = Q;  // returned even on failure, for nqg_qp_data_error
  return rc;
}

extern "C" const char *nqg_qp_data_error(const nqg_qp_data *Q) { return Q ? Q->error.c_str() : "null handle"; }

extern "C" int nqg_qp_data_sizes(const nqg_qp_data *Q, int *n, int *meq, int *mineq, int64_t *nnz) {
  if (!Q) return NQG_ERR_ARG;
  if (n) *n = Q->n;
  if (meq) *meq = Q->A.m;
  if (mineq) *mineq = Q->C.m;
  if (nnz) {
    nnz[0] = (int64_t)Q->H.i.size();
    nnz[1] = (int64_t)Q->A.i.size();
    nnz[2] = (int64_t)Q->C.i.size();
  }
  return NQG_OK;
}

extern "C" int nqg_qp_data_export(const nqg_qp_data *Q, int *Hp, int *Hi, double *Hx, double *q, int *Ap, int *Ai,
                                  double *Ax, double *b, int *Cp, int *Ci, double *Cx, double *d) {
  if (!Q) return NQG_ERR_ARG;
  auto cp = [](const auto &v, auto *dst) {
    if (dst) std::copy(v.begin(), v.end(), dst);
  };
  cp(Q->H.p, Hp), cp(Q->H.i, Hi), cp(Q->H.x, Hx), cp(Q->q.v, q);
  cp(Q->A.p, Ap), cp(Q->A.i, Ai), cp(Q->A.x, Ax), cp(Q->b.v, b);
  cp(Q->C.p, Cp), cp(Q->C.i, Ci), cp(Q->C.x, Cx), cp(Q->d.v, d);
  return NQG_OK;
}

extern "C" int nqg_qp_data_extras(const nqg_qp_data *Q, double *fixed, double *optimal_obj, int *n_primals,
                                  double *primals, int *n_duals, double *duals) {
  if (!Q) return NQG_ERR_ARG;
  if (fixed) *fixed = Q->fixed;
  if (optimal_obj) *optimal_obj = Q->optimal_obj;
  if (n_primals) *n_primals = (int)Q->primals.v.size();
  if (primals) std::copy(Q->primals.v.begin(), Q->primals.v.end(), primals);
  if (n_duals) *n_duals = (int)Q->duals.v.size();
  if (duals) std::copy(Q->duals.v.begin(), Q->duals.v.end(), duals);
  return NQG_OK;
}

extern "C" const char *nqg_qp_data_description(const nqg_qp_data *Q) { return Q ? Q->description.c_str() : ""; }

extern "C" int nqg_qp_data_destroy(nqg_qp_data *Q) {
  delete Q;
  return NQG_OK;
}
