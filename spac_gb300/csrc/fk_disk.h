// Pseudospectral disk rows: the GPU replacement for SpAc's
// PseudoespectralCirculoSolver (Solvers/PseudoespectralCirculoSolver.cpp:2-260)
// and Interpolador_PS::Interpola (BVP/Interpolador_PS.cpp:34-61).
//
// The reference builds, per disk, the dense (N2+1) N_c collocation matrix of
// the polar Laplacian plus c (N_c equispaced angles x N2+1 Chebyshev radii,
// outer ring replaced by identity rows), factors it by full-pivot Householder
// QR and solves it for the right-hand side of B and for the Fourier cardinal
// function of every periphery node; each solution is interpolated at the
// disk's interior nodes.
//
// Every block of that matrix is circulant in the angle (identity, the
// half-turn shift of the mirrored radius, the periodic second derivative), so
// with constant c the operator splits exactly into N_c/2 + 1 real (N2+1)^2
// systems, one per Fourier mode k:
//   M_k = A1 + (-1)^k A2 + mu_k diag(1/r^2) + c I   (row 0: identity)
// with A1 = D1 + R E1, A2 = D2 + R E2 the radial Chebyshev blocks and mu_k the
// eigenvalues of the periodic second-derivative matrix.  A solve is a real
// DFT in the angle, one small matrix-vector product per mode and the inverse
// DFT.  When c varies over the disk, M_k uses its mean c_bar and the solve
// iterates z <- L0^-1 (rhs - (c - c_bar) z) (Richardson on the constant-c
// operator); it converges because |c - c_bar| R^2 is small next to the
// disk's first Dirichlet eigenvalue (5.78 on the unit disk), and an
// iteration cap turns divergence into an error instead of a wrong answer.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>

namespace fk {

struct BvpDev;

constexpr int kDiskMaxCircle = 128;  // N_circunferencia
constexpr int kDiskMaxRadial = 63;   // N_radio: (N_radio + 1) / 2 <= 32 radii
constexpr int kDiskMaxPeriph = 128;  // periphery nodes
constexpr int kDiskMaxIter = 100;    // Richardson iterations when c varies

// One disk solve (PseudoespectralCirculoSolver::Inicializa + Resuelve).
struct DiskHost {
  double cx = 0, cy = 0, radius = 0, theta0 = 0;
  int n_circle = 0, n_radial = 0;
  std::vector<double> periph_theta;  // nudos_periferia[i].posicion_angular
  std::vector<double> inner_xy;      // nudos_interior[p].posicion_cartesiana
  std::vector<int> inner_row;        // assembly: CSR row of each interior node
  std::vector<int> csr_pos;          // assembly: n_inner x n_periph CSR positions
};

struct DiskDev {
  double cx, cy, radius, theta0;
  int nc, half, n_periph, n_inner;
  long long tab_off;    // radial class: r[half], A1[half^2], A2[half^2], r2inv[half], bw[2 half], diam[2 half]
  long long mu_off;     // mu_k, k = 0 .. nc/2
  long long grid_off;   // c and -f at the grid points, 2 x nc*half
  long long minv_off;   // (nc/2 + 1) x half x half
  long long z_off;      // (n_periph + 1) solutions of zstride doubles
  long long zstride;    // max(nc*half, 2 (nc/2 + 1) half): grid values or spectrum
  long long inner_off;  // first interior node of the disk (in the batch)
  long long g_off;      // first G entry (n_inner x n_periph)
  long long periph_off; // first periphery angle
};

// Host-side batch: tables shared by disks of equal (radius, N_radio) and N_c.
struct DiskBatch {
  std::vector<DiskDev> disks;
  std::vector<double> tab, periph_theta, inner_xy;
  std::vector<int> inner_disk, inner_row, csr_pos;
  long long grid_total = 0, minv_total = 0, z_total = 0, g_total = 0, n_inner = 0;
  int max_nc = 0, max_half = 0, max_rhs = 0, max_modes = 0;
  bool has_csr = false;
};

// Validates the disks and fills the batch (radial operators, mode
// eigenvalues, offsets).  False with a message on invalid sizes.
bool disk_prepare(const std::vector<DiskHost>& in, DiskBatch& out, std::string& err);

struct DiskArgs {
  const BvpDev* bvp;         // the problem (device)
  const DiskDev* disks;
  int n_disks;
  const double* tab;
  const double* periph_theta;
  const double* inner_xy;
  const int* inner_disk;     // disk of every interior node
  double* grid;              // workspace: grid_total doubles
  double* cbar;              // workspace: per disk mean c ([d]) ...
  int* varying;              // ... and whether c varies over it
  double* minv;              // workspace: minv_total
  double* z;                 // workspace: z_total
  double* G;                 // out: g_total (may be null)
  double* B;                 // out: n_inner (may be null)
  const int* inner_row;      // assembly scatter (null: none)
  const int* csr_pos;
  double* val;
  double* Bcsr;
  int* flags;                // [0] singular mode matrix, [1] no convergence
};

// Launches the four disk kernels on `s`; ev (4 events, may be null) marks
// start, after the solves, after the interpolation.
cudaError_t disk_launch(int problem, const DiskArgs& a, const DiskBatch& b, cudaStream_t s, cudaEvent_t* ev);

}  // namespace fk
