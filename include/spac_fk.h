/* spac_fk.h -- C ABI of the GB300 Feynman-Kac solver (libspac_fk.so).
 *
 * The GPU replacement for SpAc's FeynmanKacSolver node and point solves and
 * for the G/B scatter into SistemaLineal.  Plain C types only; every call
 * returns an int status (FK_OK = 0, negative on error; the message is in
 * fk_last_error).  No exception crosses the ABI and there is no CPU fallback:
 * without a usable CUDA device fk_create fails with FK_ERR_NO_DEVICE.
 *
 * Conventions
 *  - Coordinates, step sizes and outputs are double on the host side.
 *  - Output pointers may be host or device memory (checked with
 *    cudaPointerGetAttributes); device pointers are written in place on the
 *    context's stream and the call returns after the stream has drained.
 *  - Random numbers: counter-based Philox4x32-10.  Path p of item i in a call
 *    with stream id s uses counter (step, p, i, s) and key (seed lo, seed hi);
 *    the stream id advances by one after every solve call unless set with
 *    fk_set_stream.  Results are therefore reproducible for a given seed and
 *    call sequence, independent of the launch shape.
 *  - Step loop: a path is stopped after max_steps steps (fk_set_max_steps,
 *    default 2^24); such paths are counted in fk_stats.n_capped and make the
 *    call return FK_ERR_STEP_CAP after all outputs are written.
 */
#ifndef SPAC_FK_H
#define SPAC_FK_H
#ifdef __cplusplus
extern "C" {
#endif

#define FK_OK 0
#define FK_ERR_ARG (-1)
#define FK_ERR_CUDA (-2)
#define FK_ERR_REGISTRY (-3)
#define FK_ERR_STEP_CAP (-4)
#define FK_ERR_NOT_FOUND (-5)
#define FK_ERR_NO_DEVICE (-6)
#define FK_ERR_CAPACITY (-7)
#define FK_ERR_NUMERIC (-8)   /* a disk solve met a singular mode matrix or did not converge */

/* BVP coefficient sets compiled as fused device functors.  Each is the GPU
 * twin of a set of reference coefficient function pointers (BVP/BVP.hpp:17-28):
 *  FK_PROBLEM_FRANKE   BVPs/Franke_Poisson.hpp:4-73 (u, g, c = 0, f = -Lap u,
 *                      sigma = 1.41421356237 I, b = 0, F = -sigma^T grad u)
 *  FK_PROBLEM_MONEGROS BVPs/Monegros_Revamped.hpp:4-75 (c = -1)
 *  FK_PROBLEM_ANISO    sigma sigma^T = 2(1 + 0.5 sin 2pi x sin 2pi y) I,
 *                      b = (y - 1/2, 1/2 - x), c = -(1 + x^2 + y^2),
 *                      u = Franke (1 + x y), f = -(L u)
 *  FK_PROBLEM_DISK     Franke rescaled to the disk (prob = cx, cy, R):
 *                      u(x) = Franke((x - c)/(2R) + 1/2), sigma = 1.41421356237 I
 *  FK_PROBLEM_ROBIN    FK_PROBLEM_ANISO with reflecting rectangle sides: the
 *                      reflecting step Paso_Reflejante (Solvers/FeynmanKacSolver.cpp:19-67)
 *                      where Frontera::Absorbente is false (BVP/Frontera.hpp:23-36).
 *                      prob[0] = side mask (1: x = x0, 2: y = y0, 4: x = x1, 8: y = y1),
 *                      prob[1] = varphi (Y += varphi Y dL), prob[2] = rho (the
 *                      reflecting step runs within rho of the side); psi =
 *                      d_n u - varphi u (Z += psi Y dL), so u is the exact solution.
 *  FK_PROBLEM_MONEGROS_POISSON  BVPs/Monegros_Poisson.hpp:4-74 (the Monegros u
 *                      with c = 0, f = -Lap u: the problem of main_test_mpi.cpp) */
enum {
  FK_PROBLEM_FRANKE = 0,
  FK_PROBLEM_MONEGROS = 1,
  FK_PROBLEM_ANISO = 2,
  FK_PROBLEM_DISK = 3,
  FK_PROBLEM_ROBIN = 4,
  FK_PROBLEM_MONEGROS_POISSON = 5
};
/* Frontera distance functors: Dominios/Rectangulo.hpp:7-229 (x0,y0,x1,y1) and
 * Dominios/Circulo.hpp:7-22 (r,cx,cy). */
enum { FK_SHAPE_RECT = 0, FK_SHAPE_CIRCLE = 1 };
/* Control variate term xi += Y F(X).dW (FeynmanKacSolver.cpp:14):
 * none (F = 0, the reference default), exact (F = -sigma^T grad u), or a
 * learned MLP (F = -sigma^T grad u_hat). */
enum { FK_CV_NONE = 0, FK_CV_EXACT = 1, FK_CV_MLP = 2 };
/* Arithmetic of the path stepping; per-node sums are FP64 in both. */
enum { FK_FP64 = 0, FK_FP32 = 1 };

typedef struct fk_ctx fk_ctx;

typedef struct {
  int problem;      /* FK_PROBLEM_* */
  int cv;           /* FK_CV_* */
  int dom_shape;    /* FK_SHAPE_* of frontera_dominio */
  double dom[4];    /* its parameters */
  double prob[4];   /* problem parameters (FK_PROBLEM_DISK: cx, cy, R) */
  int mlp_id;       /* FK_CV_MLP: network from fk_mlp_create */
} fk_bvp_desc;

/* Per-solve statistics: the public members of FeynmanKacSolver after Update()
 * (Solvers/FeynmanKacSolver.hpp:80-83, FeynmanKacSolver.cpp:294-323), with the
 * reference's xi/xixi slot aliasing reproduced, followed by plain extras. */
typedef struct {
  double phi, phiphi, phi_VR, phiphi_VR, xi, xixi, xiphi, APL, RNGC;
  double B;             /* node solves: averaged B (Update(Nudo&), :324-334) */
  double n_paths;
  double n_domain_exits;
  double n_capped;
  double xi_mean;       /* true E[xi] and E[xi^2] */
  double xi_sq_mean;
  double mean_steps;
} fk_stats;

/* Reference arc (Mesh/Interfaz.hpp:14-37): nodes on a circle arc with the
 * inverse-multiquadric-in-theta RBF stencil (Interfaz.cpp:206-264). */
typedef struct {
  double cx, cy, radius, c2;
  int interior;          /* arc code of Interfaz::Inicia_Cuadrado */
  int n;                 /* nodes on the arc */
  const double* theta;   /* n node angles (posicion_angular) */
  const int* gids;       /* n global node ids (indice_global) */
  const double* iPsi;    /* n*n column-major inverse of Psi, or NULL: computed
                            on the GPU in FP64 (full-pivot Gauss-Jordan) */
} fk_arc_desc;

/* One node solve (Solve_OMP_Analytic(Nudo&, N, h, rho, BVP, Interfaz)). */
typedef struct {
  double x, y;           /* Nudo::posicion_cartesiana */
  double h;              /* time step */
  unsigned paths;        /* numero_trayectorias */
  int frontera;          /* Nudo::frontera: B = g(x), no paths */
  int row;               /* Nudo::indice_global (CSR row) */
  int stencil;           /* arc id (fk_register_arc) */
} fk_node_item;

/* ---- context ------------------------------------------------------------ */
int fk_create(fk_ctx** ctx, int device, unsigned long long seed);
int fk_destroy(fk_ctx* ctx);
const char* fk_last_error(const fk_ctx* ctx);
int fk_set_stream(fk_ctx* ctx, unsigned stream_id);
int fk_get_stream(const fk_ctx* ctx, unsigned* stream_id);
int fk_set_max_steps(fk_ctx* ctx, int max_steps);
/* Launch shape of the path kernel: threads per block and paths per work
 * chunk (0 = autotuned / default). */
int fk_set_launch(fk_ctx* ctx, int block_threads, int chunk_paths);
/* Limits of the kernels' bounded waits, in seconds (0 restores the default).
 * slot_wait_s: a path-kernel warp's wait for a chunk slot that another warp
 * of its CTA is still refilling (default 60 s + 1 us x max_steps, far above
 * any real wait, which the step cap bounds); barrier_s: a CTA's wait at a
 * grid barrier of the persistent MLP trainer (default 5 s).  A wait that runs
 * out ends its kernel early and the call returns FK_ERR_CUDA ("... timed
 * out"); the context stays usable, and that call's outputs (or the network's
 * parameters, for a training call) are incomplete.  No reference
 * counterpart: the reference has no waits between threads. */
int fk_set_wait_limits(fk_ctx* ctx, double slot_wait_s, double barrier_s);
/* cudaStream_t of the context, as void* */
int fk_cuda_stream(const fk_ctx* ctx, void** stream);
/* Device time (ms, CUDA events on the context stream) of the kernels of the
 * last solve: [0] path kernel, [1] finalize/scatter kernel, [2] launches. */
int fk_last_timing(const fk_ctx* ctx, double out[3]);
/* Stencil windows of the last patch-stencil solve whose moments were formed
 * into G rows (summed over items and, in adaptive rounds, over chunks): the
 * G/B scatter's work, 20 moments per window.  No reference counterpart (a
 * measurement). */
int fk_last_windows(const fk_ctx* ctx, long long* windows);

/* ---- problem registry (BVP) ---------------------------------------------- */
int fk_register_bvp(fk_ctx* ctx, const fk_bvp_desc* desc, int* bvp_id);

/* ---- point solves: Solve_OMP_Analytic(X0, N, h, rho, BVP)
 *      (Solvers/FeynmanKacSolver.cpp:335-342), n points in one launch.
 *      sub_shape/sub_params (4 per point) may be NULL: subdomain = domain. */
int fk_solve_points(fk_ctx* ctx, int bvp_id, int n, const double* xy, const unsigned* paths,
                    const double* h, const int* sub_shape, const double* sub_params,
                    int precision, fk_stats* out);

/* Batched uneven point solves: n points, each of its own registered BVP
 * (all of one problem functor and control mode), path count and step size,
 * in ONE persistent launch: chunks of every point's paths are handed to the
 * CTAs longest-first and finished paths are regenerated at once, so points
 * with 1e3 and 1e5 paths and different h share the grid without idling.
 * No reference counterpart beyond Solve_OMP_Analytic(X0,...) called per point. */
int fk_solve_points_multi(fk_ctx* ctx, int n, const int* bvp_ids, const double* xy, const unsigned* paths,
                          const double* h, int precision, fk_stats* out);
/* Autotuner of the persistent launch: times the path kernel (CUDA events) on
 * the given batched solve with every path count scaled by sample_fraction,
 * for block sizes {64, 128, 256} x chunk sizes {512, 2048, 8192, 32768}, and
 * keeps the fastest pair in the context (as fk_set_launch).  The tuning runs
 * do not advance the context's random stream id. */
int fk_autotune_points(fk_ctx* ctx, int n, const int* bvp_ids, const double* xy, const unsigned* paths,
                       const double* h, int precision, double sample_fraction, int* best_block, int* best_chunk,
                       double* best_ms);

/* ---- point solves without any allocation ----------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they solve: embedders that reserve all device memory up front
 * and forbid later allocations (a framework's caching allocator owns the GPU),
 * and real-time hosts that cannot afford an allocation's latency or the
 * device synchronisation it may imply.  Same kernels and random stream as
 * fk_solve_points (point i, path p uses the Philox counter
 * (step, p, i, stream_id) under key seed), and every point's paths are
 * split into chunks over the whole grid as there; no fk_ctx is needed.
 * d_xy (2n doubles), d_paths (n), d_h (n) and d_out (n fk_stats) are device
 * buffers owned by the caller; launches go on `cuda_stream` (a cudaStream_t,
 * NULL = default stream) of the current device and are not synchronised.
 * Scratch memory is one 4 MiB static device array per GPU that loads the
 * library, held until the process exits; n > FK_NOALLOC_MAX_POINTS returns
 * FK_ERR_CAPACITY.  The first call in a CUDA context (per device, and again
 * after cudaDeviceReset) looks up the array's device address, so make it
 * before any stream capture.  All calls share the array: calls whose kernels
 * overlap on the GPU race and give wrong results.  FK_CV_MLP is not accepted
 * (the learned control variate needs a context's network): FK_ERR_ARG.
 * Errors found by the kernels are not returned (the call does not wait for
 * them): a point solved completely has d_out[i].n_paths == d_paths[i] and
 * d_out[i].n_capped == 0; a smaller n_paths means the kernel gave up on some
 * of the point's paths, and n_capped counts paths stopped at max_steps. */
#define FK_NOALLOC_MAX_POINTS 16384
int fk_solve_points_noalloc(const fk_bvp_desc* bvp, unsigned long long seed, unsigned stream_id, int n,
                            const double* d_xy, const unsigned* d_paths, const double* d_h, int precision,
                            int max_steps, void* cuda_stream, fk_stats* d_out);

/* ---- node solves on reference arcs --------------------------------------- */
int fk_register_arc(fk_ctx* ctx, const fk_arc_desc* arc, int* arc_id);
/* the arc's iPsi as used by the kernels (n*n column-major) */
int fk_arc_ipsi(fk_ctx* ctx, int arc_id, double* iPsi);
/* Batched Solve_OMP_Analytic(Nudo&, ...) (FeynmanKacSolver.cpp:344-355):
 * G receives, for item k, the arc's n averaged G entries at offset
 * sum_{j<k} n(items[j].stencil); B[k] the averaged B; stats may be NULL. */
int fk_solve_nodes_arc(fk_ctx* ctx, int bvp_id, int n_items, const fk_node_item* items,
                       int precision, double* G, double* B, fk_stats* stats);

/* ---- meshes and batched G/B assembly -------------------------------------- */
/* Malla::Construye_Cuadrado (Mesh/Malla.cpp:12-83): circles on a grid, FK
 * items for the interior nodes of perimeter circles (main_test_serial.cpp:54-62). */
int fk_mesh_circles(fk_ctx* ctx, const double dom[4], int n_side, double superposicion,
                    double theta0, int nodes_per_circle, double c2_corner, double c2_side,
                    int* mesh_id);
/* Square patches (no reference counterpart): n_sub x n_sub subdomains of
 * [x0,x1]x[y0,y1], each enlarged by `enlarge` times its width on every side;
 * nodes_per_side equispaced nodes on each patch side inside the domain; one FK
 * item per (node, patch strictly containing it); exit values by a Gaussian
 * RBF (phi = exp(-(eps r)^2), eps = eps_spacing / node spacing) on the `knn`
 * nearest nodes of the exit patch's boundary. */
int fk_mesh_square_patches(fk_ctx* ctx, const double dom[4], int n_sub, int nodes_per_side,
                           double enlarge, double eps_spacing, int knn, int* mesh_id);
typedef struct {
  int n_rows, nnz, n_items, n_nodes, n_stencils, max_stencil;
  double spacing;        /* square patches: node spacing along a side */
} fk_mesh_info;
int fk_mesh_get_info(fk_ctx* ctx, int mesh_id, fk_mesh_info* info);
/* node table: xy[2*n_nodes]; flags[n_nodes] (bit0 = frontera) */
int fk_mesh_nodes(fk_ctx* ctx, int mesh_id, double* xy, int* flags);
/* items: row[n_items], xy[2*n_items], stencil[n_items], frontera[n_items] */
int fk_mesh_items(fk_ctx* ctx, int mesh_id, int* row, double* xy, int* stencil, int* frontera);
/* stencil s: node ids (global rows) of its nodes, count returned in *n */
int fk_mesh_stencil_nodes(fk_ctx* ctx, int mesh_id, int s, int* gids, int* n);
/* The k-window of the Gaussian exit stencil that the path kernel picks for a
 * point (x, y) on the boundary of patch s of a square-patch mesh: the
 * window's first chain node (*window; the window is k consecutive chain
 * nodes, modulo the chain length on a closed patch), the point's nearest
 * node on its side (*nearest), and how an exit there visits the window's
 * nodes (*walk: bits 0-1 FP32 stepping, bits 2-3 FP64; 0 every node, 1 outward
 * from the nearest node to the first node beyond the weight cutoff, 2 a fixed
 * range of +-2 (FP32) or +-4 (FP64) chain places around it).  Evaluated on
 * the host in FP64 with the kernel's window table.  Introspection of the
 * stencil; no reference counterpart. */
int fk_mesh_window(fk_ctx* ctx, int mesh_id, int s, double x, double y, int* window, int* nearest, int* walk);
/* SistemaLineal::Inicializa_CSR (Mesh/SistemaLineal.cpp:39-66): sorted CSR
 * pattern, diagonal = number of containing patches, placeholder 1e-23. */
int fk_mesh_csr(fk_ctx* ctx, int mesh_id, int* rowptr, int* col, double* val0);
/* Assemble: paths per item (or per-item array `paths_per_item` if non-NULL),
 * time step h.  Writes val (CSR values = pattern + sum of item G rows, as
 * SistemaLineal::Actualiza_GB, Mesh/SistemaLineal.cpp:68-88) and B; item_G /
 * item_B / item_stats (optional, NULL to skip) receive per-item results. */
int fk_assemble(fk_ctx* ctx, int mesh_id, int bvp_id, unsigned paths, const unsigned* paths_per_item,
                double h, int precision, double* val, double* B, double* item_G, double* item_B,
                fk_stats* item_stats);

/* ---- adaptive assembly in rounds ------------------------------------------
 * For path counts chosen per item from the estimates so far (an SE target),
 * with the path sums kept on the device between rounds: the reference solves
 * each node once with a fixed N (Solve_OMP_Analytic, FeynmanKacSolver.cpp:344-355,
 * then SistemaLineal::Actualiza_GB, Mesh/SistemaLineal.cpp:68-88); running it
 * again with more paths and averaging by hand would keep only averages.
 *  fk_assembly_begin  zeroes the mesh's running sums (square-patch meshes).
 *  fk_assembly_round  runs paths_per_item[i] more paths of item i (0 = none)
 *                     with BVP bvp_of_item[i] (NULL: bvp_id for every item;
 *                     one problem functor per round, and items with a learned
 *                     control variate share one network, so learned-CV items
 *                     and their plain fallback share one launch), and ADDS
 *                     their sums -- each chunk's unnormalised G row, B and the
 *                     statistics -- to the running sums on the device.
 *                     item_var (may be NULL) receives each item's per-path
 *                     variance of phi_VR over this round's paths.  Every round
 *                     uses the context's next random stream id and the same h.
 *  fk_assembly_end    forms every item's path-weighted G row and B from the
 *                     running sums (the same as one run of all its paths:
 *                     G = -(sum over all paths of Y w(X_tau)) / N) and writes
 *                     them as fk_assemble does; item_stats are over all
 *                     rounds' paths.  It may be called after any round (the
 *                     sums stay until the next fk_assembly_begin). */
int fk_assembly_begin(fk_ctx* ctx, int mesh_id);
int fk_assembly_round(fk_ctx* ctx, int mesh_id, int bvp_id, const int* bvp_of_item, const unsigned* paths_per_item,
                      double h, int precision, double* item_var);
int fk_assembly_end(fk_ctx* ctx, int mesh_id, double* val, double* B, double* item_G, double* item_B,
                    fk_stats* item_stats);

/* ---- pseudospectral disk rows ---------------------------------------------
 * PseudoespectralCirculoSolver::Inicializa(centro, radio, N_circunferencia,
 * N_radio, theta_0, BVP) + Resuelve(BVP, nudos_interior, nudos_periferia)
 * (Solvers/PseudoespectralCirculoSolver.cpp:2-189, :215-260) with
 * Interpolador_PS::Interpola (BVP/Interpolador_PS.cpp:34-61): the
 * deterministic FP64 rows of the interior nodes of a disk, against the
 * disk's periphery nodes.  The collocation system (Laplacian in polar
 * coordinates + c, outer ring = identity rows; sigma and b of the BVP are not
 * used, as in the reference) is solved on the GPU per Fourier mode; with a
 * c that varies over the disk the solve iterates on the constant-c operator
 * and returns FK_ERR_NUMERIC if that does not converge. */
typedef struct {
  double cx, cy, radius;
  double theta0;               /* angle of the first grid ray (nudos_circunferencia[0].posicion_angular) */
  int n_circle;                /* N_circunferencia: grid angles, even, 2..128 */
  int n_radial;                /* N_radio: Chebyshev intervals on a diameter, odd, 3..63 */
  int n_periph;                /* periphery nodes (nudos_periferia), 2..128 */
  const double* periph_theta;  /* their posicion_angular */
  int n_inner;                 /* interior nodes (nudos_interior) */
  const double* inner_xy;      /* their posicion_cartesiana, (x, y) pairs */
} fk_disk_desc;
/* Batched disk solves.  For disk d, G receives n_inner x n_periph entries
 * (row-major, nudos_interior[p].G[periphery i]) at offset sum of the earlier
 * disks' n_inner * n_periph, and B the n_inner values nudos_interior[p].B at
 * offset sum of the earlier n_inner.  fk_last_timing: [0] grid, mode and
 * solve kernels, [1] interpolation kernel, [2] launches. */
int fk_solve_disks_ps(fk_ctx* ctx, int bvp_id, int n_disks, const fk_disk_desc* disks, double* G, double* B);
/* Circle meshes: n_radial > 0 makes fk_assemble also fill the rows of the
 * interior nodes of every full (non-perimeter) circle by the disk solve
 * with N_radio = n_radial, added into val and B as
 * SistemaLineal::Actualiza_GB(Interfaz&) (Mesh/SistemaLineal.cpp:90-95), as
 * the reference drivers do (main_test_serial.cpp:67-80); 0 switches it off. */
int fk_mesh_set_disk_solver(fk_ctx* ctx, int mesh_id, int n_radial);

/* ---- host-side consumers of the assembled system (no GPU needed) -----------
 * Restarted GMRES(restart) with right Jacobi preconditioning on a CSR system,
 * to check an assembled solution on the host.  Replaces, for checking only,
 * SistemaLinealSolverGMRES::Resuelve (Solvers/SistemaLinealSolverGMRES.hpp:157-597,
 * METIS + MUMPS Schwarz preconditioner over MPI).  x holds the initial guess.
 * Returns FK_ERR_NOT_FOUND if the relative residual stays above 10 tol. */
int fk_gmres_csr(int n, const int* rowptr, const int* col, const double* val, const double* b, double* x, double tol,
                 int max_iter, int restart, int* iters, double* rel_resid);
/* The same GMRES with a choice of right preconditioner: FK_PC_JACOBI
 * (diag(A)^-1, as fk_gmres_csr) or FK_PC_ILU0 (incomplete LU on A's own
 * sparsity pattern; each row's columns ascending with its diagonal present,
 * as the assembled CSR patterns are, else FK_ERR_ARG; FK_ERR_NUMERIC on a
 * zero pivot). */
enum { FK_PC_JACOBI = 0, FK_PC_ILU0 = 1 };
int fk_gmres_csr_pc(int n, const int* rowptr, const int* col, const double* val, const double* b, double* x,
                    double tol, int max_iter, int restart, int precond, int* iters, double* rel_resid);
/* The reference's text formats (values in C++ general format, as its
 * setf(fixed, scientific) leaves them): dir/G.txt "row col value" (%.8g) and
 * dir/B.txt (%.8g) -- SistemaLineal::Escribe_GB_COO (Mesh/SistemaLineal.cpp:96-110);
 * dir/G_i.txt, G_j.txt, G_ij.txt and B.txt (%.10g) -- Escribe_GB_CSR (:124-138). */
int fk_write_gb_coo(const char* dir, int n_rows, const int* rowptr, const int* col, const double* val,
                    const double* B);
int fk_write_gb_csr(const char* dir, int n_rows, const int* rowptr, const int* col, const double* val,
                    const double* B);
/* SistemaLineal::Lee_GB_COO (Mesh/SistemaLineal.cpp:139-164): header "nnz n_rows" then
 * row-sorted "row col value" lines; call with NULL arrays for the sizes. */
int fk_read_gb_coo(const char* path, int* n_rows, int* nnz, int* rowptr, int* col, double* val);
/* Malla::Escribe_Posiciones (Mesh/Malla.cpp:99-112): "gid x y u" (%.12g) */
int fk_write_positions(const char* path, int n, const int* gids, const double* xy, const double* u);

/* ---- learned control variate ---------------------------------------------
 * No counterpart in the reference (its control-variate hook is the field F of
 * the BVP, Coeficiente_Vectorial F, set to -sigma^T grad u by hand).  One MLP
 * 2 -> 64 -> 64 -> 64 -> 1 (SiLU) per region, input mapped from the region's
 * rectangle to [-1,1]^2; BF16 weights on the tensor cores, FP32 accumulate,
 * FP32 master copy updated by Adam.  A BVP registered with cv = FK_CV_MLP and
 * mlp_id uses F = -sigma^T grad u_hat, where grad u_hat is tabulated on a
 * grid per region (fk_mlp_build_table) and interpolated bilinearly at every
 * step; paths of mesh items use the region of their stencil when the network
 * has one region per stencil, region 0 otherwise. */
int fk_mlp_create(fk_ctx* ctx, int n_regions, const double* region_rects, unsigned long long init_seed,
                  int* mlp_id);
/* parameters per region, packed W1(64x2),b1,W2(64x64),b2,W3(64x64),b3,W4(1x64),b4, row-major FP32;
 * get/set move all regions ([n_regions][n]) */
int fk_mlp_num_params(fk_ctx* ctx, int mlp_id, int* n);
int fk_mlp_get_params(fk_ctx* ctx, int mlp_id, float* params);
int fk_mlp_set_params(fk_ctx* ctx, int mlp_id, const float* params);
/* Adam on mean((u_hat - target)^2): every step draws `batch` samples (a
 * multiple of 128) per region with replacement (Philox, shuffle_seed) from
 * the samples of that region (region[i], NULL = region 0).  loss_history
 * (length steps, may be NULL) receives the mean batch loss of each step. */
int fk_mlp_train(fk_ctx* ctx, int mlp_id, int n, const double* xy, const double* target, const int* region,
                 int steps, int batch, double lr, unsigned long long shuffle_seed, float* loss_history);
/* Training kernel of fk_mlp_train:
 *  FK_TRAIN_AUTO   the grid trainer where its cooperative launch fits the device, else per-step launches;
 *  FK_TRAIN_GRID   all steps in one cooperative launch: per step the CTAs' gradient partials,
 *                  a grid barrier, Adam on each CTA's slice of the parameters (partials summed
 *                  in a fixed order), a grid barrier (FK_ERR_ARG where the launch does not fit);
 *  FK_TRAIN_STEPS  one graph-captured pass + Adam launch pair per step. */
enum { FK_TRAIN_AUTO = 0, FK_TRAIN_GRID = 1, FK_TRAIN_STEPS = 2 };
int fk_mlp_set_trainer(fk_ctx* ctx, int mlp_id, int trainer);
/* Fits the output layer (W4, b4) of every region exactly: ridge least
 * squares of the targets on the current last hidden layer over the given
 * samples (variable projection; the hidden layers stay as trained).  ridge
 * is relative to the mean diagonal of the feature Gram matrix (1e-6 is a
 * good default).  FK_ERR_NUMERIC if the regularised Gram matrix is not
 * positive definite. */
int fk_mlp_fit_output(fk_ctx* ctx, int mlp_id, int n, const double* xy, const double* target, const int* region,
                      double ridge);
/* forward + input gradient at n points: out[3*n] = (u_hat, du/dx, du/dy) */
int fk_mlp_eval(fk_ctx* ctx, int mlp_id, int n, const double* xy, const int* region, double* out);
/* loss and parameter gradient of mean((u_hat - target)^2) over all n samples, region 0 (FP32 grad) */
int fk_mlp_loss_grad(fk_ctx* ctx, int mlp_id, int n, const double* xy, const double* target,
                     double* loss, float* grad);
/* tabulates grad u_hat on a grid x grid lattice of every region (used by FK_CV_MLP solves) */
int fk_mlp_build_table(fk_ctx* ctx, int mlp_id, int grid);
/* The table of fk_mlp_build_table, as FK_CV_MLP steps interpolate it:
 * *grid = its lattice size (0 before the first build or after
 * fk_mlp_set_params); if table is not NULL it receives n_regions x grid x
 * grid FP32 pairs (du_hat/dx, du_hat/dy), the pair of lattice point (i, j) of
 * region r, at x0 + (x1 - x0) i / (grid - 1), y0 + (y1 - y0) j / (grid - 1)
 * of the region's rectangle, at table[2 ((r grid + j) grid + i)]. */
int fk_mlp_get_table(fk_ctx* ctx, int mlp_id, int* grid, float* table);

#ifdef __cplusplus
}
#endif
#endif
