/*
 * cevgpu.h -- C ABI of the GB300 (sm_103a) Yee-stencil library that replaces
 * ceviche's CPU FDFD solve and FDTD time loop.
 *
 * Conventions
 *   - Every entry point returns an int status: CEV_OK (0), < 0 error,
 *     > 0 "finished but not converged"-style outcomes.  cev_last_error_string()
 *     describes the last error of the calling thread.
 *   - Grids are (nx, ny) in C order, flat index i*ny + j (ceviche's
 *     _grid_to_vec, ceviche/fdfd.py:118-120).  A batch of problems is laid out
 *     [batch][nx][ny].
 *   - Complex arrays are interleaved (re, im): complex64 = float2,
 *     complex128 = double2.
 *   - All array arguments are DEVICE pointers unless stated otherwise; the
 *     caller owns them.  Plans own only their small coefficient tables.
 *   - Work is enqueued on the given stream; host-side validation errors come
 *     back synchronously.  cev_fdfd_solve synchronises the stream once per
 *     restart cycle to read the FP64 true residual.
 */
#ifndef CEVGPU_H_
#define CEVGPU_H_

#include <stddef.h>
#include <cuda_runtime.h>

#if defined(__GNUC__)
#define CEV_API __attribute__((visibility("default")))
#else
#define CEV_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define CEV_OK 0
#define CEV_ERR_INVALID (-1)
#define CEV_ERR_CUDA (-2)
#define CEV_ERR_WORKSPACE (-3)
#define CEV_ERR_NUMERIC (-4)
#define CEV_NOT_CONVERGED 1
#define CEV_STAGNATED 2

#define CEV_POL_EZ 0
#define CEV_POL_HZ 1

#define CEV_PREC_C64 0  /* complex64 fields, float eps   */
#define CEV_PREC_C128 1 /* complex128 fields, double eps */

#define CEV_PRECOND_NONE 0
#define CEV_PRECOND_SHIFTED_LAPLACIAN 1 /* nested-dissection factors of the shifted operator */
#define CEV_PRECOND_LEARNED 2
#define CEV_PRECOND_SEPARABLE 3 /* exact inverse of the constant-eps stretched operator */
#define CEV_PRECOND_DIRECT 4    /* nested-dissection complex64 factors of the operator */

/* Last error message of the calling thread ("" if none). */
CEV_API const char* cev_last_error_string(void);
/* Library version, major*10000 + minor*100 + patch. */
CEV_API int cev_version(void);

/* ============================== FDFD ==================================== */

typedef struct cev_fdfd_plan_s* cev_fdfd_plan;

/*
 * Precomputes the SC-PML stencil coefficient tables of `batch` problems that
 * share a grid and differ in omega.  Replaces the per-solve sparse assembly of
 * ceviche/derivatives.py:34-216 (compute_derivative_matrices, create_S_matrices,
 * create_sfactor, s_value) and ceviche/fdfd.py:80-112 (_setup_derivatives,
 * Bloch phases).  omegas is a HOST array of length batch.
 */
CEV_API int cev_fdfd_plan_create(cev_fdfd_plan* plan, int pol, int nx, int ny, int batch, double dL,
                         const double* omegas, int npml_x, int npml_y, double bloch_x,
                         double bloch_y);
CEV_API int cev_fdfd_plan_destroy(cev_fdfd_plan plan);

/*
 * Complex permittivity (lossy media; ceviche accepts a complex eps_r,
 * fdfd.py:40-44, and its complex-eps tests run forward-mode jacobians,
 * tests/test_gradients_fdfd_complex.py).  With on = 1 every FDFD entry point
 * of this plan reads eps (and deps) as interleaved complex arrays of the
 * documented precision (complex128 where double is documented, complex64 for
 * CEV_PREC_C64 apply), and geps as complex128 accumulating the PyTorch-
 * convention gradient dL/dRe(eps) + i dL/dIm(eps).  Default 0 (real eps).
 * Multi-frequency plans take a real eps only.
 */
CEV_API int cev_fdfd_plan_set_eps_complex(cev_fdfd_plan plan, int on);
/* Row scaling of the non-dimensional system the solver works on:
 * A' = scale*A with scale = mu0*dL^2 (Ez) or eps0*dL^2 (Hz). */
CEV_API double cev_fdfd_plan_scale(cev_fdfd_plan plan);

/*
 * y = A x  (transpose=1: y = A^T x) for every problem of the batch.
 * Matrix-free form of fdfd_ez._make_A / fdfd_hz._make_A
 * (ceviche/fdfd.py:172-185, 211-233) as applied by sp_mult
 * (ceviche/primitives.py:58-72); the transpose replaces the transposed-index
 * products of primitives.py:81-86, 121-135.
 * precision CEV_PREC_C64: eps is float*, x/y complex64;
 * CEV_PREC_C128: eps is double*, x/y complex128.
 * eps_shared=1: one eps grid for the whole batch, else [batch][nx][ny].
 * si_units=1 returns A x in SI units, 0 the non-dimensional A' x.
 */
CEV_API int cev_fdfd_apply(cev_fdfd_plan plan, const void* eps, int eps_shared, const void* x, void* y,
                   int transpose, int precision, int si_units, cudaStream_t stream);

typedef struct {
  double tol;         /* target FP64 true relative residual ||Ax-b||/||b|| (default 1e-6) */
  double inner_rtol;  /* residual reduction at which a complex64 inner cycle stops (1e-4) */
  int max_iters;      /* cap on Arnoldi iterations over all cycles */
  int restart;        /* Krylov dimension per cycle, 1..64 */
  int precond;        /* CEV_PRECOND_* */
  int transpose;      /* solve A^T x = b (adjoint solve) */
  int use_x0;         /* x holds an initial guess on entry */
  int reorth;         /* 1: classical Gram-Schmidt with a second pass */
  int max_stall;      /* cycles without a 10% residual drop before CEV_STAGNATED */
  int mg_levels;      /* reserved (0) */
  double mg_shift;    /* shifted-operator imaginary shift beta the caller factors with (0.5) */
  const void* learned; /* CEV_PRECOND_LEARNED: a cev_learned_precond handle */
  const void* separable; /* CEV_PRECOND_SEPARABLE: a cev_sep_precond handle */
  const void* direct;  /* CEV_PRECOND_DIRECT / _SHIFTED_LAPLACIAN: a cev_nd_precond handle */
} cev_solve_opts;

typedef struct {
  int status;      /* CEV_OK, CEV_NOT_CONVERGED, CEV_STAGNATED, CEV_ERR_NUMERIC */
  int iterations;  /* Arnoldi iterations spent on this problem */
  int cycles;      /* restart cycles (= FP64 residual evaluations - 1) */
  int reserved;
  double residual; /* final FP64 true relative residual */
  double bnorm;    /* ||b|| (SI) */
} cev_solve_info;

/*
 * Separable preconditioner (CEV_PRECOND_SEPARABLE).  With eps replaced by a
 * constant c per problem, the stretched operator of a plan is separable:
 *   Ez: A'_c = -(Tx (x) I + I (x) Ty) - k2 c,   Hz: A'_c = (Tx (x) I + I (x) Ty)/(c + 1e-5) + k2
 * (k2 = eps0 mu0 w^2 dL^2; Tx, Ty the plan's 1D stencil operators, see
 * cev_fdfd_axis_matrix).  With Tx = Vx Lx Vx^-1 and Ty = Vy Ly Vy^-1 its
 * inverse is (Vx (x) Vy) diag(1/d) (Vx^-1 (x) Vy^-1): four dense complex
 * GEMMs per application (strided-batched over the problems) and one
 * scaling kernel.  Used as the right preconditioner of flexible GMRES; the
 * solve still converges on the true operator to the FP64 residual.
 * vx, vxi: complex128 [batch][nx][nx] (row-major Vx, Vx^-1); vy, vyi:
 * [batch][ny][ny]; dinv: complex128 [batch][nx][ny] = 1/d (complex128
 * because the PML makes the 1D eigenbases ill-conditioned).  All device
 * pointers, owned by the caller and kept alive with the handle.  transpose
 * states which operator (A or A^T) the factors belong to; a solve uses the
 * handle only with the same transpose flag.
 */
typedef struct cev_sep_precond_s* cev_sep_precond;
CEV_API int cev_sep_precond_create(cev_sep_precond* out, cev_fdfd_plan plan, int transpose,
                                   const void* vx, const void* vxi, const void* vy,
                                   const void* vyi, const void* dinv);
CEV_API int cev_sep_precond_destroy(cev_sep_precond h);

/*
 * Direct preconditioner (CEV_PRECOND_DIRECT): a nested-dissection multifrontal
 * factorisation of the plan's non-dimensional operator A' (or A'^T with
 * transpose = 1) for eps (double [1 or batch][nx][ny], real or, with
 * cev_fdfd_plan_set_eps_complex, complex), in complex64 and without the
 * periodic wrap entries; the separators are eliminated in their dissection
 * order, with partial pivoting only inside each block of up to 32 pivots
 * (which leaves the factorisation's sparsity unchanged).  It stands where
 * ceviche factors the
 * assembled matrix with SuperLU (ceviche/solvers.py:50-62, reached from
 * primitives.py:103-119); here the factors precondition flexible GMRES and the
 * FP64 true residual still decides convergence, so the complex64 rounding and
 * the dropped wrap only cost iterations.  The separators split the longer
 * side of each box; fronts are dense and swept by Gauss-Jordan, so applying
 * M^-1 is GEMVs.  shift > 0 factors the shifted operator (mass term times
 * 1 - i*shift), the exact complex-shifted-Laplacian inverse that
 * CEV_PRECOND_SHIFTED_LAPLACIAN uses.  The handle owns its factors (about
 * 80-110 complex64 numbers per cell and problem; cev_nd_precond_info) and
 * keeps a pointer to the plan, which must outlive it.  create synchronises
 * the stream; it returns CEV_ERR_NUMERIC for a zero or non-finite pivot
 * (a pivot block that is singular even with pivoting).
 * apply: z = M^-1 v for every problem (complex64 [batch][nx][ny]).
 */
typedef struct cev_nd_precond_s* cev_nd_precond;
CEV_API int cev_nd_precond_create(cev_nd_precond* out, cev_fdfd_plan plan, const double* eps,
                                  int eps_shared, int transpose, double shift,
                                  cudaStream_t stream);
CEV_API int cev_nd_precond_apply(cev_nd_precond h, const void* v, void* z, cudaStream_t stream);
CEV_API int cev_nd_precond_info(cev_nd_precond h, size_t* factor_bytes, double* factor_cmacs,
                                int* depths);
CEV_API int cev_nd_precond_destroy(cev_nd_precond h);
/* Host-side analysis of the nested-dissection tree of an nx x ny grid (no
 * CUDA call): tree nodes, depths, complex64 factor entries and Gauss-Jordan
 * complex multiply-adds per problem, original-entry count, and cover[2] =
 * (cells eliminated - nx*ny, sum of their ids - sum of 0..nx*ny-1), both 0
 * when every cell is eliminated exactly once. */
CEV_API int cev_nd_analyse(int nx, int ny, size_t* n_nodes, int* depths, size_t* factor_elems,
                           double* factor_cmacs, size_t* n_desc, long long* cover);

/*
 * Learned preconditioner (CEV_PRECOND_LEARNED).  A 4-level convolutional
 * encoder-decoder (base width c0: c0 -> 8*c0 channels, bf16 activations,
 * fp32 accumulation on the tensor cores) that maps a Krylov basis vector of a
 * single-frequency Ez plan to an approximation of A'^-1 v.  It has no
 * counterpart in ceviche: it is the right preconditioner of the flexible
 * GMRES that replaces ceviche's direct solve (ceviche/solvers.py:37-62).
 *
 * Parameters are one fp32 device vector of cev_learned_param_count(c0)
 * numbers: per conv layer W[cout][cin][3][3] then b[cout], then the 1x1
 * head W[2][c0], b[2].  The caller owns parameters, gradients and the Adam
 * state; the handle owns the packed bf16 weights and the activations for
 * max_batch problems of nx x ny (both divisible by 8).
 *
 * forward: z = |r| f(r/|r|, eps, k2) for every problem of the plan (r, z
 *   complex64 [batch][nx][ny]; eps float [batch][nx][ny] or shared).
 * backward: grad += dL/dparams for dL/dz = gz (complex64, d/dRe + i d/dIm),
 *   through the activations of the last forward.
 * cev_adam_step: one Adam update of n parameters (step counts from 1).
 */
typedef struct cev_learned_precond_s* cev_learned_precond;
CEV_API int cev_learned_param_count(int c0, size_t* count);
CEV_API int cev_learned_create(cev_learned_precond* out, int nx, int ny, int max_batch, int c0);
CEV_API int cev_learned_set_params(cev_learned_precond h, const float* params, cudaStream_t stream);
CEV_API int cev_learned_forward(cev_learned_precond h, cev_fdfd_plan plan, const float* eps,
                                int eps_shared, const void* r, void* z, cudaStream_t stream);
CEV_API int cev_learned_backward(cev_learned_precond h, const void* gz, float* grad,
                                 cudaStream_t stream);
CEV_API int cev_adam_step(float* p, const float* g, float* m, float* v, size_t n, float lr,
                          float beta1, float beta2, float eps, int step, cudaStream_t stream);
/* Convolution kernels: 1 = tcgen05 with TMEM accumulators (default; layers
 * with <= 32 input channels run a persistent variant), 2 = tcgen05 without
 * the persistent variant, 0 = mma.sync.  cev_learned_tc_fault reads and clears the flag the tcgen05
 * kernel sets when one of its bounded waits ran out (synchronises). */
CEV_API int cev_learned_set_conv_impl(int impl);
CEV_API int cev_learned_tc_fault(int* fault);
CEV_API int cev_learned_destroy(cev_learned_precond h);

/*
 * The plan's 1D stencil operator along one axis (0 = x, 1 = y) for problem b
 * and the forward (transpose = 0) or transposed tables, as a dense host
 * matrix (n x n complex128, row-major, interleaved): row i holds cm at
 * column i-1, cp at i+1 and -(am + ap) at i (indices mod n, Bloch phasors
 * on the wrap), the non-dimensional derivative part of fdfd.py:172-233
 * along that axis.  No CUDA call.
 */
CEV_API int cev_fdfd_axis_matrix(cev_fdfd_plan plan, int b, int axis, int transpose, double* out);

/* Fills opts with the defaults documented above. */
CEV_API void cev_solve_opts_default(cev_solve_opts* opts);

/* Bytes of device workspace cev_fdfd_solve needs for these options. */
CEV_API size_t cev_fdfd_solve_workspace_size(cev_fdfd_plan plan, const cev_solve_opts* opts);

/*
 * Solves A x = b (or A^T x = b) for every problem of the batch to the FP64
 * true relative residual opts->tol with restarted (flexible) GMRES: complex64
 * Arnoldi cycles on the GPU, each restart an FP64 residual b - A x and an FP64
 * update of x (mixed-precision iterative refinement).  Replaces
 * ceviche/primitives.py:103-119 sp_solve -> ceviche/solvers.py:37-62
 * solve_linear/_solve_direct (and fills the _solve_cuda stub, solvers.py:77-79).
 * eps: double [1 or batch][nx][ny]; b, x: complex128 [batch][nx][ny] in SI
 * units (b = 1j*omega*J as built by fdfd.py:189, 237).
 * info: HOST array of `batch` records.  Returns the worst per-problem status.
 */
CEV_API int cev_fdfd_solve(cev_fdfd_plan plan, const double* eps, int eps_shared, const void* b, void* x,
                   const cev_solve_opts* opts, cev_solve_info* info, void* workspace,
                   size_t workspace_bytes, cudaStream_t stream);

/*
 * Secondary fields from the solved component, complex128, SI units.
 * Ez: (f1, f2) = (Hx, Hy) = (-Dyb Ez, Dxb Ez)/(1j*omega*mu0)   (fdfd.py:138-147)
 * Hz: (f1, f2) = (Ex, Ey) = (Dyf Hz/(eps_xx+1e-5), -Dxf Hz/(eps_yy+1e-5))/(1j*omega*eps0)
 *     (fdfd.py:150-162, averages of fdfd.py:200-209)
 */
CEV_API int cev_fdfd_fields(cev_fdfd_plan plan, const double* eps, int eps_shared, const void* fz,
                    void* f1, void* f2, cudaStream_t stream);

/*
 * Reverse mode of cev_fdfd_fields (PyTorch cotangent convention,
 * g = dL/dRe + i dL/dIm): gz += M1^H g1 + M2^H g2.  For Hz the direct
 * dependence of (Ex, Ey) on eps is added to geps (double, same batch layout as
 * eps; summed over the batch when eps_shared).  Restates the sp_mult x-VJP
 * (ceviche/primitives.py:81-86) used through fdfd.py:138-162.
 */
CEV_API int cev_fdfd_fields_adjoint(cev_fdfd_plan plan, const double* eps, int eps_shared, const void* fz,
                            const void* g1, const void* g2, void* gz, double* geps,
                            cudaStream_t stream);

/*
 * geps += dL/d(eps) contributed by the system matrix, given the forward
 * solution x and mu = A^{-T} conj(g_x) (the transposed solve of the cotangent).
 * Ez: Re(mu * eps0*omega^2 * x); Hz: chain through 1/(eps_yy+1e-5),
 * 1/(eps_xx+1e-5) and the averages.  Restates grad_sp_solve_entries_reverse
 * (ceviche/primitives.py:121-128) chained to eps by fdfd.py:179 / 211-233.
 */
CEV_API int cev_fdfd_grad_eps(cev_fdfd_plan plan, const double* eps, int eps_shared, const void* x,
                      const void* mu, double* geps, cudaStream_t stream);

/*
 * Forward mode (JVP).  rhs += -(dA/d eps . deps) x, the right-hand side of the
 * tangent solve A dx = i w dsrc - dA x.  Restates
 * grad_sp_solve_entries_forward / grad_sp_mult_entries_forward
 * (ceviche/primitives.py:90-98, 139-146) chained from eps through
 * fdfd.py:179 (Ez) and fdfd.py:211-233 (Hz).  deps has the layout of eps.
 */
CEV_API int cev_fdfd_jvp_rhs(cev_fdfd_plan plan, const double* eps, int eps_shared,
                             const double* deps, const void* x, void* rhs, cudaStream_t stream);

/*
 * Direct eps tangent of the secondary fields: (df1, df2) += d(F1, F2)/d eps . deps
 * at fixed Fz.  Zero for Ez; for Hz the 1/(eps_avg + 1e-5) factors of
 * fdfd.py:150-162.  The full tangent adds cev_fdfd_fields(dFz).
 */
CEV_API int cev_fdfd_fields_jvp(cev_fdfd_plan plan, const double* eps, int eps_shared,
                                const double* deps, const void* fz, void* df1, void* df2,
                                cudaStream_t stream);

/*
 * Multi-frequency (time-modulated) Ez FDFD, ceviche/fdfd.py:247-359
 * (fdfd_mf_ez).  The plan holds M = 2*nsb+1 sidebands W_m = omega + m*omega_mod
 * (m = -nsb..nsb) sharing the centre-frequency PML tables; fields and sources
 * are complex128 [M][nx][ny].  The modulation of harmonic k (k < nfreq) is
 * given as c_k = delta_k * exp(1j*phi_k), complex128 [nfreq][nx][ny]:
 *   A_mm = -(1/mu0)(Dxf Dxb + Dyf Dyb) - eps0 W_m^2 eps,
 *   A_m,m+k+1 = -eps0/2 W_m^2 c_k,   A_m,m-k-1 = -eps0/2 W_m^2 conj(c_k).
 * cev_fdfd_fields / cev_fdfd_fields_adjoint apply per sideband with W_m
 * (fdfd.py:339-355).  Destroy with cev_fdfd_plan_destroy.
 */
CEV_API int cev_fdfd_mf_plan_create(cev_fdfd_plan* plan, int nx, int ny, double dL, double omega,
                                    double omega_mod, int nsb, int npml_x, int npml_y,
                                    double bloch_x, double bloch_y);
/* y = A x or A^T x of the coupled system, complex128, SI units. */
CEV_API int cev_fdfd_mf_apply(cev_fdfd_plan plan, const double* eps, int nfreq,
                              const void* coupling, const void* x, void* y, int transpose,
                              cudaStream_t stream);
CEV_API size_t cev_fdfd_mf_solve_workspace_size(cev_fdfd_plan plan, int nfreq,
                                                const cev_solve_opts* opts);
/* Solves the coupled system (one Krylov problem of M*nx*ny unknowns); info: 1 record.
 * Replaces sp_solve of fdfd_mf_ez._solve_fn (fdfd.py:328-337). */
CEV_API int cev_fdfd_mf_solve(cev_fdfd_plan plan, const double* eps, int nfreq,
                              const void* coupling, const void* b, void* x,
                              const cev_solve_opts* opts, cev_solve_info* info, void* workspace,
                              size_t workspace_bytes, cudaStream_t stream);
/*
 * Gradients through A given x and mu = A^{-T} conj(g): geps (double [nx][ny])
 * += dL/d eps; gcoupling (complex128 [nfreq][nx][ny], may be NULL) += dL/dc_k
 * in the PyTorch convention.  Restates the sp_solve entries VJP
 * (ceviche/primitives.py:121-128) chained through fdfd.py:289-326.
 */
CEV_API int cev_fdfd_mf_grad(cev_fdfd_plan plan, int nfreq, const void* x, const void* mu,
                             double* geps, void* gcoupling, cudaStream_t stream);

/* ======================= generic sparse (CSR) ============================ */
/*
 * y = A x for a complex128 CSR matrix (n x n, nnz entries, int32 indices):
 * sp_mult of ceviche/primitives.py:58-72 for entries/indices that are not a
 * Yee stencil.  The caller builds CSR from COO with duplicates summed
 * (ceviche/utils.py:13-25); A^T is applied by passing the transpose's CSR.
 */
CEV_API int cev_csr_apply(int n, int nnz, const int* row_ptr, const int* col, const void* val,
                          const void* x, void* y, cudaStream_t stream);
CEV_API size_t cev_csr_solve_workspace_size(int n, int nnz, const cev_solve_opts* opts);
/*
 * x = A^{-1} b (sp_solve, ceviche/primitives.py:103-119) with the same
 * mixed-precision restarted GMRES as cev_fdfd_solve, on the scaled system
 * (scale*A) x = scale*b; pass scale ~ 1/max|A_ij| so the complex64 cycle
 * stays in range.  info: 1 record.
 */
CEV_API int cev_csr_solve(int n, int nnz, const int* row_ptr, const int* col, const void* val,
                          double scale, const void* b, void* x, const cev_solve_opts* opts,
                          cev_solve_info* info, void* workspace, size_t workspace_bytes,
                          cudaStream_t stream);

/* ---------------------------------------------------------------- probes
 * Replaces the per-step host loop of ceviche.utils.measure_fields
 * (ceviche/utils.py:316-332): out[t*out_stride + p] = sum_q weight[q] *
 * field[t*field_stride + cell[q]] for q in probe_ptr[p] .. probe_ptr[p+1]-1,
 * t = 0 .. nrows-1, accumulated in FP64 (deterministic).  field is float32
 * (field_is_f64 = 0) or float64; probe_ptr has n_probe + 1 entries; nrows <= 65535. */
CEV_API int cev_probe_measure(int n_probe, const int* probe_ptr, const int* cell, const double* weight,
                              const void* field, int field_is_f64, int nrows, long long field_stride,
                              double* out, long long out_stride, cudaStream_t stream);

/* ----------------------------------------------------------------- modes
 * Replaces ceviche.modes.get_modes (ceviche/modes.py:10-45) and the
 * shift-invert ARPACK call behind it (solver_eigs, modes.py:68-78): for each
 * of `batch` cross sections eps[b][0..n-1] (double, device), the m eigenpairs
 * of A = diag(eps) + Dxf Dxb / k0^2 (k0 = omega / C_0; the (n, 1)-grid SC-PML
 * derivatives of derivatives.py with npml cells per side and a periodic wrap)
 * nearest sigma = max(eps), nearest first.  Outputs (device): vals complex128
 * [batch][m] (n_eff^2), vecs complex128 [batch][m][n] with unit 2-norm and
 * the largest-magnitude entry real positive (the reference's phase is
 * ARPACK's, arbitrary), iters / status int [batch] (0 converged to tol, 1 not
 * converged after max_iters, 2 singular shift).  n >= 3, 1 <= m <= min(n, 24).
 * Synchronises the stream before returning. */
CEV_API size_t cev_mode_workspace_size(int batch, int n, int m);
CEV_API int cev_mode_solve(int batch, int n, const double* eps, double omega, double dL, int npml, int m,
                           double tol, int max_iters, void* vals, void* vecs, int* iters, int* status,
                           void* workspace, size_t workspace_bytes, cudaStream_t stream);

/* Host-side eigen-decomposition of a small dense complex matrix (k <= 24;
 * the Rayleigh-Ritz step of cev_mode_solve, exported for checking): h, w, v
 * are interleaved complex128 host arrays, h and v row-major k x k, column j of
 * v the unit eigenvector of w[j].  No CUDA call. */
CEV_API int cev_dense_eig(int k, const double* h, double* w, double* v);

/* ============================== FDTD ==================================== */

typedef struct cev_fdtd_plan_s* cev_fdtd_plan;

/*
 * 2D (Nz = 1) Yee FDTD with ceviche's integrated-sigma PML.
 * Replaces ceviche/fdtd.py:12-72 (construction, setters), 213-316 (dt,
 * sigmas, update coefficients).  precision: CEV_PREC_C64 -> float32 fields,
 * CEV_PREC_C128 -> float64 fields.  eps: DEVICE double [nx][ny].
 * A plan's buffers (tables, 1/eps, the runners' shadow state and exchange
 * flags) come from the device's default stream-ordered memory pool, which
 * keeps up to 256 MB of freed blocks for reuse, so plans created and
 * destroyed in a loop allocate without a driver call; they are allocated on
 * `stream` and usable on it at once.  cev_fdtd_plan_destroy waits for the
 * device before returning the buffers to the pool.
 */
CEV_API int cev_fdtd_plan_create(cev_fdtd_plan* plan, int nx, int ny, double dL, int npml_x, int npml_y,
                         int precision, const double* eps, cudaStream_t stream);
CEV_API int cev_fdtd_plan_destroy(cev_fdtd_plan plan);
/* Replaces the eps_r setter's coefficient refresh (fdtd.py:63-72). */
CEV_API int cev_fdtd_set_eps(cev_fdtd_plan plan, const double* eps, cudaStream_t stream);
/* dt of fdtd.py:213-222. */
CEV_API double cev_fdtd_dt(cev_fdtd_plan plan);

/*
 * Caller-owned field state (device arrays of nx*ny float or double each).
 * TM: hx, hy, dz + PML integrals icex, icey, idz.
 * TE: hz, dx, dy + PML integrals ihz, ichx, ichy.
 * The curl integrals are stored without the 1/dL factor of fdtd.py:85-117.
 */
typedef struct {
  void* hx; void* hy; void* dz; void* icex; void* icey; void* idz;
  void* hz; void* dx; void* dy; void* ihz; void* ichx; void* ichy;
} cev_fdtd_state;

/*
 * One reference time step (fdtd.py:74-144) with dense sources jx, jy, jz
 * (device arrays in the field precision, NULL = no source).  te != 0 also
 * updates the TE fields.
 */
CEV_API int cev_fdtd_step(cev_fdtd_plan plan, const cev_fdtd_state* st, const void* jx, const void* jy,
                  const void* jz, int te, cudaStream_t stream);

/*
 * E fields from the D state: ez = dz/eps_zz (TM); ex = dx/eps_xx, ey = dy/eps_yy (TE)
 * (fdtd.py:134-142, averages of ceviche/utils.py:153-176).  NULL outputs are skipped.
 */
CEV_API int cev_fdtd_e_fields(cev_fdtd_plan plan, const cev_fdtd_state* st, void* ex, void* ey, void* ez,
                      cudaStream_t stream);

/* Sparse source J(t) = w_k * amps[t] at cells idx_k, and point probes. */
typedef struct {
  int n_src;
  const int* src_idx;   /* device, flat cell indices */
  const void* src_w;    /* device, field precision */
  const void* amps;     /* device, field precision, amps[t - t_begin] */
  int n_probe;
  const int* probe_idx; /* device, flat cell indices */
  void* probe_out;      /* device, field precision, [nsteps][n_probe] Ez after each step */
} cev_fdtd_io;

/*
 * nsteps TM steps with sparse source and probes, time-blocked: each launch
 * advances a tile by several steps in shared memory.  Bitwise the same
 * recurrence as cev_fdtd_step.
 */
CEV_API int cev_fdtd_run_tm(cev_fdtd_plan plan, const cev_fdtd_state* st, int nsteps,
                    const cev_fdtd_io* io, cudaStream_t stream);

/* Sparse TE sources J(t) = (wx, wy) * amps[t] at cells idx_k, and Hz probes. */
typedef struct {
  int n_src;
  const int* src_idx;   /* device, flat cell indices */
  const void* src_wx;   /* device, field precision: Jx weight per source cell */
  const void* src_wy;   /* device, field precision: Jy weight per source cell */
  const void* amps;     /* device, field precision, amps[t - t_begin] */
  int n_probe;
  const int* probe_idx; /* device, flat cell indices */
  void* probe_out;      /* device, field precision, [nsteps][n_probe] Hz after each step */
} cev_fdtd_io_te;

/*
 * nsteps TE steps (Hz, Dx, Dy with Jx, Jy sources: the TE half of
 * ceviche/fdtd.py:79-137 with Nz = 1), time-blocked like cev_fdtd_run_tm
 * (K = 8 steps per launch on 32 x 48 tiles; per-step kernels on grids below
 * one tile region).  Bitwise the same recurrence as cev_fdtd_step with te = 1
 * and dense Jx = wx * amps[t], Jy = wy * amps[t].
 */
CEV_API int cev_fdtd_run_te(cev_fdtd_plan plan, const cev_fdtd_state* st, int nsteps,
                            const cev_fdtd_io_te* io, cudaStream_t stream);

/*
 * Allocation-free variant of cev_fdtd_run_tm.  No counterpart in the
 * reference.  For callers that cannot allocate device memory (a host
 * framework that owns every device allocation, or a real-time loop in which
 * cudaMalloc/cudaFree must not be called): it needs no plan and calls no
 * cudaMalloc, cudaFree or allocating library routine.  Its tables, 1/eps and
 * the shadow copy of the double-buffered state live in a static device array
 * that every GPU loading this library keeps until the process exits
 * (7 MiB + 512 KiB).  float32 state (the fields of a CEV_PREC_C64 plan);
 * eps is device double [nx][ny]; nx*ny <= 262144 and nx, ny <= 8192, larger
 * grids are rejected with CEV_ERR_INVALID.  The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress); make that first call
 * before any stream capture.  Every call shares the array, so calls that
 * overlap on the GPU (other streams, other host threads) race.  A call
 * enqueues kernels (its PML tables are computed on the device) and
 * device-to-device copies only; it copies nothing from host memory.
 */
CEV_API int cev_fdtd_run_tm_noalloc(int nx, int ny, double dL, int npml_x, int npml_y,
                                    const double* eps, const cev_fdtd_state* st, int nsteps,
                                    const cev_fdtd_io* io, cudaStream_t stream);

/*
 * Reverse of ONE TM step of cev_fdtd_step.  On entry adj holds dL/d(state after the step) (hx, hy, dz, icex, icey, idz)
 * and g_ez (optional, with dz_out = Dz after the step) dL/dEz after the step;
 * on return adj holds dL/d(state before the step) and geps (double [nx][ny])
 * has the step's eps term added.  dz_in = Dz before the step.  scratch: 4*nx*ny
 * elements of the field precision.  The step's source gradient dL/dJz is
 * the gradient of Dz after the step (g_dz + g_ez/eps), which the caller forms
 * before the call.  This is the per-step VJP that autograd tapes through
 * ceviche/fdtd.py:74-144 for test_gradients_fdtd.py:66-165.
 */
CEV_API int cev_fdtd_step_adjoint_tm(cev_fdtd_plan plan, const void* dz_in, const void* dz_out,
                                     const void* g_ez, const cev_fdtd_state* adj, void* scratch,
                                     double* geps, cudaStream_t stream);

/* Workspace bytes for cev_fdtd_adjoint_tm. */
CEV_API size_t cev_fdtd_adjoint_workspace_size(cev_fdtd_plan plan, int nsteps, int ckpt_every);

/*
 * Reverse-time adjoint of a TM run from zero fields: for the loss
 * L = sum_t sum_p w[t][p] * Ez_t(probe_p) (w: device [nsteps][n_probe], field
 * precision) adds dL/d(eps) to geps (device double [nx][ny]).  The forward
 * run is checkpointed every ckpt_every steps and recomputed per segment.
 * Replaces the autograd tape over fdtd.forward used by
 * tests/test_gradients_fdtd.py:66-165.
 */
CEV_API int cev_fdtd_adjoint_tm(cev_fdtd_plan plan, int nsteps, int ckpt_every, const cev_fdtd_io* io,
                        const void* w, double* geps, void* workspace, size_t workspace_bytes,
                        cudaStream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* CEVGPU_H_ */
