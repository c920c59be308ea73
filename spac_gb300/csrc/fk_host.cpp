// Host-side consumers of the assembled system: a restarted GMRES to check the
// assembled solution (the reference solves with METIS + MUMPS Schwarz GMRES
// over MPI, Solvers/SistemaLinealSolverGMRES.hpp:157-597; here a plain
// single-process GMRES(m) with a Jacobi or ILU(0) preconditioner), and the
// reference's text formats for G, B and the node positions.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/spac_fk.h"

namespace {

void spmv(int n, const int* rp, const int* col, const double* val, const double* x, double* y) {
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int k = rp[i]; k < rp[i + 1]; ++k) s += val[k] * x[col[k]];
    y[i] = s;
  }
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

std::string join(const char* dir, const char* name) {
  std::string d(dir ? dir : ".");
  if (!d.empty() && d.back() != '/') d += '/';
  return d + name;
}

// Right preconditioners of the GMRES: apply(v, out) = M^-1 v.
struct Precond {
  int kind = FK_PC_JACOBI;
  int n = 0;
  const int* rp = nullptr;
  const int* col = nullptr;
  std::vector<double> dinv;  // Jacobi: diag(A)^-1
  std::vector<double> lu;    // ILU(0): L (unit, below the diagonal) and U on A's pattern
  std::vector<int> diag;     // position of each row's diagonal
  std::vector<double> y;

  // Jacobi: M = diag(A).  ILU(0): M = L U with L and U restricted to A's
  // sparsity (the IKJ elimination dropping every fill-in entry); needs each
  // row's columns ascending with the diagonal present.
  int setup(int kind_, int n_, const int* rp_, const int* col_, const double* val) {
    kind = kind_;
    n = n_;
    rp = rp_;
    col = col_;
    if (kind == FK_PC_JACOBI) {
      dinv.assign(n, 1.0);
      for (int i = 0; i < n; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k)
          if (col[k] == i && val[k] != 0.0) dinv[i] = 1.0 / val[k];
      return FK_OK;
    }
    if (kind != FK_PC_ILU0) return FK_ERR_ARG;
    diag.assign(n, -1);
    for (int i = 0; i < n; ++i)
      for (int k = rp[i]; k < rp[i + 1]; ++k) {
        if (k > rp[i] && col[k] <= col[k - 1]) return FK_ERR_ARG;  // columns not ascending
        if (col[k] < 0 || col[k] >= n) return FK_ERR_ARG;
        if (col[k] == i) diag[i] = k;
      }
    for (int i = 0; i < n; ++i)
      if (diag[i] < 0) return FK_ERR_ARG;
    lu.assign(val, val + rp[n]);
    std::vector<int> pos(n, -1);
    for (int i = 0; i < n; ++i) {
      for (int k = rp[i]; k < rp[i + 1]; ++k) pos[col[k]] = k;
      for (int k = rp[i]; k < diag[i]; ++k) {  // l_ik for the columns left of the diagonal, in order
        const int c = col[k];
        const double piv = lu[diag[c]];
        if (piv == 0.0) return FK_ERR_NUMERIC;
        const double l = lu[k] / piv;
        lu[k] = l;
        for (int q = diag[c] + 1; q < rp[c + 1]; ++q) {  // row i -= l_ik (U row c), on row i's pattern
          const int p = pos[col[q]];
          if (p >= 0) lu[p] -= l * lu[q];
        }
      }
      for (int k = rp[i]; k < rp[i + 1]; ++k) pos[col[k]] = -1;
      if (lu[diag[i]] == 0.0) return FK_ERR_NUMERIC;
    }
    y.assign(n, 0.0);
    return FK_OK;
  }

  void apply(const double* v, double* out) {
    if (kind == FK_PC_JACOBI) {
      for (int i = 0; i < n; ++i) out[i] = dinv[i] * v[i];
      return;
    }
    for (int i = 0; i < n; ++i) {  // L y = v
      double s = v[i];
      for (int k = rp[i]; k < diag[i]; ++k) s -= lu[k] * y[col[k]];
      y[i] = s;
    }
    for (int i = n - 1; i >= 0; --i) {  // U out = y
      double s = y[i];
      for (int k = diag[i] + 1; k < rp[i + 1]; ++k) s -= lu[k] * out[col[k]];
      out[i] = s / lu[diag[i]];
    }
  }
};

}  // namespace

extern "C" {

int fk_gmres_csr_pc(int n, const int* rowptr, const int* col, const double* val, const double* b, double* x,
                    double tol, int max_iter, int restart, int precond, int* iters, double* rel_resid) {
  if (n < 1 || !rowptr || !col || !val || !b || !x || restart < 1 || max_iter < 1 || !(tol > 0)) return FK_ERR_ARG;
  Precond M;
  int rc = M.setup(precond, n, rowptr, col, val);
  if (rc) return rc;
  const int m = restart;
  std::vector<double> r(n), w(n), z(n), t(n), bnrm_v(b, b + n);
  const double bnrm = std::sqrt(dot(bnrm_v, bnrm_v));
  const double ref = bnrm > 0 ? bnrm : 1.0;
  std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
  std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1);
  int it = 0;
  double res = 0.0;
  while (it < max_iter) {
    spmv(n, rowptr, col, val, x, w.data());
    for (int i = 0; i < n; ++i) r[i] = b[i] - w[i];
    double beta = std::sqrt(dot(r, r));
    res = beta / ref;
    if (res <= tol) break;
    for (int i = 0; i < n; ++i) V[0][i] = r[i] / beta;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m && it < max_iter; ++j, ++it) {
      M.apply(V[j].data(), z.data());
      spmv(n, rowptr, col, val, z.data(), w.data());
      for (int k = 0; k <= j; ++k) {  // modified Gram-Schmidt
        const double hk = dot(w, V[k]);
        H[k * m + j] = hk;
        for (int i = 0; i < n; ++i) w[i] -= hk * V[k][i];
      }
      const double hn = std::sqrt(dot(w, w));
      H[(j + 1) * m + j] = hn;
      if (hn > 0)
        for (int i = 0; i < n; ++i) V[j + 1][i] = w[i] / hn;
      for (int k = 0; k < j; ++k) {  // Givens rotations
        const double tk = cs[k] * H[k * m + j] + sn[k] * H[(k + 1) * m + j];
        H[(k + 1) * m + j] = -sn[k] * H[k * m + j] + cs[k] * H[(k + 1) * m + j];
        H[k * m + j] = tk;
      }
      const double a = H[j * m + j], c = H[(j + 1) * m + j];
      const double d = std::sqrt(a * a + c * c);
      cs[j] = d > 0 ? a / d : 1.0;
      sn[j] = d > 0 ? c / d : 0.0;
      H[j * m + j] = d;
      H[(j + 1) * m + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      res = std::fabs(g[j + 1]) / ref;
      if (res <= tol || hn == 0.0) { ++j; ++it; break; }
    }
    // back substitution and update x += M^{-1} V y
    std::vector<double> y(j, 0.0);
    for (int k = j - 1; k >= 0; --k) {
      double s = g[k];
      for (int q = k + 1; q < j; ++q) s -= H[k * m + q] * y[q];
      y[k] = H[k * m + k] != 0 ? s / H[k * m + k] : 0.0;
    }
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int k = 0; k < j; ++k) s += V[k][i] * y[k];
      t[i] = s;
    }
    M.apply(t.data(), z.data());
    for (int i = 0; i < n; ++i) x[i] += z[i];
    if (res <= tol) break;
  }
  // true residual
  spmv(n, rowptr, col, val, x, w.data());
  for (int i = 0; i < n; ++i) r[i] = b[i] - w[i];
  res = std::sqrt(dot(r, r)) / ref;
  if (iters) *iters = it;
  if (rel_resid) *rel_resid = res;
  return res <= tol * 10 ? FK_OK : FK_ERR_NOT_FOUND;
}

int fk_gmres_csr(int n, const int* rowptr, const int* col, const double* val, const double* b, double* x, double tol,
                 int max_iter, int restart, int* iters, double* rel_resid) {
  return fk_gmres_csr_pc(n, rowptr, col, val, b, x, tol, max_iter, restart, FK_PC_JACOBI, iters, rel_resid);
}

int fk_write_gb_coo(const char* dir, int n_rows, const int* rowptr, const int* col, const double* val, const double* B) {
  // SistemaLineal::Escribe_GB_COO (Mesh/SistemaLineal.cpp:96-110): "row col value".  The
  // reference's setf(std::ios::fixed, std::ios::scientific) clears the float field, so
  // values come out in general format with 8 significant digits (%.8g), as here.
  if (!rowptr || !col || !val || !B || n_rows < 0) return FK_ERR_ARG;
  FILE* fg = std::fopen(join(dir, "G.txt").c_str(), "w");
  FILE* fb = std::fopen(join(dir, "B.txt").c_str(), "w");
  if (!fg || !fb) {
    if (fg) std::fclose(fg);
    if (fb) std::fclose(fb);
    return FK_ERR_ARG;
  }
  for (int r = 0; r < n_rows; ++r) {
    std::fprintf(fb, "%.8g\n", B[r]);
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) std::fprintf(fg, "%d %d %.8g\n", r, col[k], val[k]);
  }
  std::fclose(fg);
  std::fclose(fb);
  return FK_OK;
}

int fk_write_gb_csr(const char* dir, int n_rows, const int* rowptr, const int* col, const double* val, const double* B) {
  // SistemaLineal::Escribe_GB_CSR (Mesh/SistemaLineal.cpp:124-138): G_i, G_j, G_ij and B,
  // values in general format with 10 significant digits (%.10g)
  if (!rowptr || !col || !val || !B || n_rows < 0) return FK_ERR_ARG;
  FILE* fi = std::fopen(join(dir, "G_i.txt").c_str(), "w");
  FILE* fj = std::fopen(join(dir, "G_j.txt").c_str(), "w");
  FILE* fv = std::fopen(join(dir, "G_ij.txt").c_str(), "w");
  FILE* fb = std::fopen(join(dir, "B.txt").c_str(), "w");
  if (!fi || !fj || !fv || !fb) {
    for (FILE* f : {fi, fj, fv, fb})
      if (f) std::fclose(f);
    return FK_ERR_ARG;
  }
  for (int r = 0; r < n_rows; ++r) {
    std::fprintf(fi, "%d\n", rowptr[r]);
    std::fprintf(fb, "%.10g\n", B[r]);
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      std::fprintf(fj, "%d\n", col[k]);
      std::fprintf(fv, "%.10g\n", val[k]);
    }
  }
  for (FILE* f : {fi, fj, fv, fb}) std::fclose(f);
  return FK_OK;
}

int fk_read_gb_coo(const char* path, int* n_rows, int* nnz, int* rowptr, int* col, double* val) {
  // SistemaLineal::Lee_GB_COO (Mesh/SistemaLineal.cpp:139-164): header "nnz n_rows",
  // then "row col value" lines sorted by row.  With rowptr/col/val NULL only
  // the sizes are returned.
  if (!path || !n_rows || !nnz) return FK_ERR_ARG;
  FILE* f = std::fopen(path, "r");
  if (!f) return FK_ERR_ARG;
  int nz = 0, nr = 0;
  if (std::fscanf(f, "%d %d", &nz, &nr) != 2 || nz < 0 || nr < 0) {
    std::fclose(f);
    return FK_ERR_ARG;
  }
  *nnz = nz;
  *n_rows = nr;
  if (!rowptr || !col || !val) {
    std::fclose(f);
    return FK_OK;
  }
  for (int i = 0; i <= nr; ++i) rowptr[i] = 0;
  int r, c, k = 0, prev = -1;
  double v;
  while (k < nz && std::fscanf(f, "%d %d %lf", &r, &c, &v) == 3) {
    if (r < 0 || r >= nr || r < prev) {
      std::fclose(f);
      return FK_ERR_ARG;
    }
    for (int q = prev + 1; q <= r; ++q) rowptr[q] = k;
    prev = r;
    col[k] = c;
    val[k] = v;
    ++k;
  }
  for (int q = prev + 1; q <= nr; ++q) rowptr[q] = k;
  std::fclose(f);
  return k == nz ? FK_OK : FK_ERR_ARG;
}

int fk_write_positions(const char* path, int n, const int* gids, const double* xy, const double* u) {
  // Malla::Escribe_Posiciones (Mesh/Malla.cpp:99-112): "gid x y u", general format, 12 significant digits
  if (!path || n < 0 || !gids || !xy || !u) return FK_ERR_ARG;
  FILE* f = std::fopen(path, "w");
  if (!f) return FK_ERR_ARG;
  for (int i = 0; i < n; ++i) std::fprintf(f, "%d %.12g %.12g %.12g\n", gids[i], xy[2 * i], xy[2 * i + 1], u[i]);
  std::fclose(f);
  return FK_OK;
}

}  // extern "C"
