// Krylov solver state shared by the solver and the preconditioners.
#pragma once

#include <functional>

#include "fdfd_plan.hpp"

namespace cev {

// Per-problem scalars of the batched GMRES, finalised on the device.
struct KState {
  double bnorm;    // ||b'|| of the non-dimensional system
  double beta;     // FP64 true residual norm at the start of the cycle
  double res_est;  // Givens estimate of the current residual norm
  double thresh;   // cycle stops when res_est <= thresh
  int active;      // Arnoldi work enabled for this problem
  int ncols;       // Krylov columns accumulated in the cycle
  int iters;       // total Arnoldi iterations
  int nan;         // non-finite value seen
  int done;        // host decided the problem is finished
  int fault;       // a bounded device wait timed out (fused cycle)
  int pad[2];
  double rscale;   // the complex64 copy of the residual is stored divided by this
};

// Device pointers of the solver workspace.
struct KCtx {
  KState* st;
  double* partial;      // [B][part_stride] cross-block partial sums
  size_t part_stride;
  unsigned* counter;    // [B][2] arrival counters (self-resetting)
  double2* H;           // [B][m][m+1] Hessenberg columns (rotated into R)
  double* cs;           // [B][m] Givens cosines
  double2* sn;          // [B][m] Givens sines
  double2* gam;         // [B][m+1] rotated residual vector
  double* sc;           // [B][m+1] 1/||v_k|| (basis stored unnormalised)
  double2* y;           // [B][m] least-squares solution
  double2* hpass;       // [B][m+1] projections of the current pass
  double* fpart;        // fused cycle: per-block partials
  unsigned* bar;        // fused cycle: grid barrier words (count, generation, fault)
  double tol, inner_rtol;
  int max_iters;
};

// ------------------------------------------------------- generic driver
// A Krylov problem: B independent systems of n unknowns each, stored
// [B][n] (complex128 x and b in the caller's units).
struct KrylovProblem {
  int B = 1;
  size_t n = 0;
  size_t res_blocks = 1;   // most blocks a residual kernel uses per problem
  size_t extra_bytes = 0;  // operator scratch at the start of the workspace
};

struct KLayout {
  size_t extra, V, Z, partial, counter, st, H, cs, sn, gam, sc, y, hpass, fpart, pc, total;
  size_t part_stride;
  int nblk;
};
KLayout klayout(const KrylovProblem& P, const cev_solve_opts& o, size_t pc_bytes);

// Operator hooks.  residual(): launch r = b' - A' x in FP64 for every problem,
// write r / KState.rscale (complex64) into V_0 and finish the reduction with
// residual_finish.  matvec(j, in, use_scale, out): out = A' (s in) with
// s = sc[b][j] when use_scale.  b' = bscale * b is the system the cycle sees.
struct KrylovOps {
  std::function<int(const KCtx&, float2* V0, cudaStream_t)> residual;
  std::function<int(const KCtx&, int j, const float2* in, int use_scale, float2* out,
                    cudaStream_t)> matvec;
  std::function<int(const KCtx&, int j, const float2* v, float2* z, cudaStream_t)> precond;
  // Optional: the whole Arnoldi cycle of an unpreconditioned small batch in
  // one launch (replaces the per-iteration matvec / dot / update launches).
  std::function<int(const KCtx&, float2* V, cudaStream_t)> cycle;
  double bscale = 1.0;
  // The preconditioner costs far more than a host round trip: after every
  // Arnoldi step the driver reads the problems' activity and ends the cycle
  // once none is left (a converging direct preconditioner needs few steps).
  bool check_each_step = false;
};

// Fused stencil cycle for small batches (cycle.cu).
struct CycArgs {
  int nx, ny, rows, m, reorth, tiles_y, units;
  int B, gp;      // problems, blocks per problem
  size_t N;
  size_t eps_bs;    // eps batch stride in elements (0: shared)
  const void* eps;  // float or float2 (complex eps)
  const Coef<float>* cx;
  const Coef<float>* cy;
  const float* k2;
  float2* V;  // [m+1][N]
  KCtx ctx;
};
int fused_max_blocks();
size_t cycle_stage_bytes();
// Blocks of the fused cycle for B problems on an nx x ny grid (0: not
// available), its work split and gp blocks per problem; limit > 0 caps gp.
int cycle_plan(int nx, int ny, int pol, int ceps, int B, int limit, int& rows, int& tiles_y,
               int& units, int& gp);
static constexpr int FUSED_MAX_BATCH = 16;
int cycle_launch(int pol, int ceps, int blocks, const CycArgs& a, cudaStream_t s);

int krylov_run(const KrylovProblem& P, const KrylovOps& ops, const cev_solve_opts& o,
               const double2* b, double2* x, cev_solve_info* info, void* ws, size_t ws_bytes,
               cudaStream_t s);
int validate_opts(const cev_solve_opts& o);

// Right preconditioner used by flexible GMRES: z = M^{-1} (sc_j v_j).
struct Precond {
  int kind = CEV_PRECOND_NONE;
  void* impl = nullptr;
};

size_t precond_workspace_size(const cev_fdfd_plan_s* p, const cev_solve_opts& o);
int precond_setup(Precond& pc, const cev_fdfd_plan_s* p, const cev_solve_opts& o, const float* eps32,
                  int eps_shared, void* ws, cudaStream_t s);
int precond_apply(Precond& pc, const KCtx& c, int j, int m, const float2* v, float2* z,
                  cudaStream_t s);

// TMA-staged Arnoldi matvec (csrc/stencil_tma.cu): Ez and Hz, real eps, ny % 4 == 0
bool tma_matvec_usable(const cev_fdfd_plan_s* p, bool eps_complex);
int tma_matvec(const cev_fdfd_plan_s* p, int tr, const float* eps32, int eps_shared,
               const float2* in, float2* out, const KCtx& c, int m, int j, int use_scale,
               cudaStream_t s);

// Nested-dissection factors (csrc/nd.cu): z = M^-1 (sc[b][sc_index] v) for
// the problems whose Arnoldi work is still on (st may be NULL: all).
int nd_apply(cev_nd_precond_s* h, const float2* v, float2* z, const double* sc, int sc_stride,
             int sc_index, const KState* st, cudaStream_t s);
int nd_check(const cev_nd_precond_s* h, const cev_fdfd_plan_s* p, int kind, int transpose);

namespace nn {
int learned_check(const cev_learned_precond_s* h, const cev_fdfd_plan_s* p);
int learned_forward(cev_learned_precond_s* h, const cev_fdfd_plan_s* p, const float* eps,
                    int eps_shared, const float2* r, float2* z, const double* sc, int sc_stride,
                    int sc_index, cudaStream_t s);
}  // namespace nn

}  // namespace cev
