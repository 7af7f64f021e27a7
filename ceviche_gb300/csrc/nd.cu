// Nested-dissection multifrontal factorisation of the FDFD stencil system in
// complex64: the right preconditioner CEV_PRECOND_DIRECT of flexible GMRES,
// and, built with a shift beta, the exact shifted-operator inverse behind
// CEV_PRECOND_SHIFTED_LAPLACIAN.
//
// ceviche reaches its solutions with a sparse direct solve
// (ceviche/solvers.py:50-62, scipy SuperLU).  Here the same kind of
// factorisation is a preconditioner: M = A' without the periodic wrap
// entries, factored in complex64 without pivoting; the FP64 true residual of
// the flexible GMRES decides convergence, so the complex64 rounding of the
// factors (and the dropped wrap) only adds iterations (typically 2-4 to 1e-6).
//
// Ordering.  The (nx, ny) grid is split recursively: a box splits its longer
// side at the midpoint by a one-cell separator line; boxes with both sides
// <= LEAF are eliminated whole.  A node of the tree eliminates its interior
// set I (the separator, or all cells of a leaf box) and couples to its
// boundary set B (the one-cell frame around its box, inside the grid), which
// is always a subset of ancestor separators.  The front of a node is the
// dense matrix F over [I; B]:
//   F = A'(I, I u B), A'(B, I)  +  the children's Schur complements (extend-add).
// Gauss-Jordan sweeps of the I pivots turn F into
//   [[ G = F_II^-1,  H = G F_IB ],
//    [ -K = -F_BI G,  S = F_BB - F_BI G F_IB ]]
// (the block "sweep operator").  S is the node's update matrix for its parent;
// G, H, -K are kept.  Applying M^-1 v is then GEMVs only:
//   forward (leaves first):  f = [v_I ; 0] + sum children's u,  u = f_B - K f_I
//   backward (root first):   x_I = G f_I - H x_B.
//
// Storage (per problem, complex64): the per-node row block [G | H] (nI x f,
// row-major) and -K (nB x nI); per depth, depth-major, so one depth of all
// problems is one contiguous range.  Schur complements live in two arenas
// alternating by depth parity (a node's children are one depth deeper).
//
// Kernels.  The leaves (4 x 4 boxes) need only the inverse of their 16 x 16
// interior block, one warp each.  Other fronts with f <= 128 are assembled
// and swept entirely in shared memory, one CTA per (node, problem), in blocks
// of up to 16 pivots (pivoted LU of the pivot block, triangular-solve panels,
// a register-tiled rank-16 update).  Larger fronts are assembled in global
// memory and swept in blocks of NB = 32 pivots: pivoted LU of the pivot
// block, row and column panels by triangular solves, then a rank-32 update of
// every other entry (64 x 64 tiles, FP32 FMA) that carries the flops.  Every
// update takes the right-looking LU split (F_rP U^-1)(L^-1 Pm F_Pc).  The
// apply kernels are bandwidth-bound GEMVs over the factor (a warp per small
// front, a warp per row of a large one).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "fdfd_plan.hpp"
#include "krylov.hpp"

namespace cev {
namespace nd {

constexpr int LEAF = 4;        // boxes with both sides <= LEAF are eliminated whole
constexpr int NB = 32;         // pivots per block step of the large-front path (one warp)
constexpr int SMALL_F = 128;   // fronts up to this size are swept in shared memory
constexpr int TILE = 64;       // update tile (rows x cols) of the large-front path
constexpr int GEMV_ROWS = 32;  // rows per CTA of the large-front apply GEMVs
constexpr int WPB = 8;         // warps (small fronts) per CTA of the apply kernels

// Factor storage of a small front (f <= SMALL_F) is column-major, so its
// apply runs one warp per front with a lane per row (coalesced, no
// reductions); a large front is row-major (warp per row, coalesced along the
// row, and the blocked sweep addresses rows).
struct Node {
  int nI, nB;
  int cells;         // offset in the cell list: nI interior then nB boundary cells
  int child[2];      // -1: none
  int cmap[2];       // offset in the map list: child's B cells -> positions in this front
  int desc, ndesc;   // original-entry descriptors
  int par;           // Schur arena of this node's depth (depth & 1)
  int small;         // f <= SMALL_F
  int lidx;          // large fronts: index in its depth's list of large fronts
  int po;            // large fronts: panel-scratch offset (in NB-element rows) within its depth
  long long top;     // [G | H] (nI x f), offset within one problem's factor block
  long long bl;      // -K (nB x nI)
  long long s;       // S (nB x nB, row-major) within one problem's block of arena par
  long long fv;      // front vector (f) within one problem's block
};

// A'(row cell, neighbour in direction dir) of one stencil row:
// dir 0 = diagonal, 1 = (i-1, j), 2 = (i+1, j), 3 = (i, j-1), 4 = (i, j+1).
struct Desc {
  int row, col, cell, dir;
};

// What defines the entries: the plan's float tables for one transpose flag.
struct Op {
  int pol, nx, ny;
  int eps_complex;
  size_t eps_bs;  // eps batch stride in elements (0: shared)
  const double* eps;
  const Coef<float>* cx;  // [B][nx]
  const Coef<float>* cy;  // [B][ny]
  const float* k2;        // [B]
  float shift;            // mass term times (1 - i shift)
};

struct Args {
  Op op;
  const Node* nodes;
  const int* cells;
  const int* cmap;
  const Desc* desc;
  float2* fac;
  float2* sar[2];
  float2* fv;
  int* fault;  // set when a pivot is zero or not finite
  float2* lub; // LU factors of the current pivot blocks [B][large fronts][NB][NB]
  int* lpv;    // their row permutations [B][large fronts][NB]
  float2* rb;  // L^-1 Pm F[P, :] of the current block, [B][ps_pp], NB x f per front
  float2* cb;  // F[:, P] U^-1 of the current block, [B][ps_pp], f x NB per front
  size_t n;    // cells per problem
  long long fac_pp, sa_pp[2], fv_pp;  // per-problem strides
  long long ps_pp;                    // per-problem stride of rb / cb
};

__device__ __forceinline__ float2 eps_at(const Op& o, int b, int i, int j) {
  i = (i + o.nx) % o.nx;
  j = (j + o.ny) % o.ny;
  const size_t k = (size_t)b * o.eps_bs + (size_t)i * o.ny + j;
  if (o.eps_complex) return make_float2((float)o.eps[2 * k], (float)o.eps[2 * k + 1]);
  return make_float2((float)o.eps[k], 0.f);
}

// 1/((a + b)/2 + 1e-5) in complex arithmetic (the Hz averages of fdfd.py:200-233)
__device__ __forceinline__ float2 hzd(float2 a, float2 b) {
  const float2 den = make_float2(0.5f * (a.x + b.x) + 1e-5f, 0.5f * (a.y + b.y));
  const float q = 1.0f / (den.x * den.x + den.y * den.y);
  return make_float2(den.x * q, -den.y * q);
}

// The entry of A' (the same arithmetic as stencil_column in stencil.cuh, with
// the mass term times (1 - i shift)).
__device__ float2 coef(const Op& o, int b, int cell, int dir) {
  const int i = cell / o.ny, j = cell - (cell / o.ny) * o.ny;
  const Coef<float> cx = o.cx[(size_t)b * o.nx + i];
  const Coef<float> cy = o.cy[(size_t)b * o.ny + j];
  const float k2 = o.k2[b];
  const float2 sh = make_float2(1.f, -o.shift);
  if (o.pol == POL_EZ) {
    switch (dir) {
      case 1: return make_float2(-cx.cm.x, -cx.cm.y);
      case 2: return make_float2(-cx.cp.x, -cx.cp.y);
      case 3: return make_float2(-cy.cm.x, -cy.cm.y);
      case 4: return make_float2(-cy.cp.x, -cy.cp.y);
      default: {
        const float2 d0 = cadd(cadd(cx.am, cx.ap), cadd(cy.am, cy.ap));
        const float2 m = cmul(cscale(eps_at(o, b, i, j), k2), sh);
        return csub(d0, m);
      }
    }
  }
  const float2 e = eps_at(o, b, i, j);
  switch (dir) {
    case 1: return cmul(cx.cm, hzd(eps_at(o, b, i - 1, j), eps_at(o, b, i - 2, j)));
    case 2: return cmul(cx.cp, hzd(e, eps_at(o, b, i - 1, j)));
    case 3: return cmul(cy.cm, hzd(eps_at(o, b, i, j - 1), eps_at(o, b, i, j - 2)));
    case 4: return cmul(cy.cp, hzd(e, eps_at(o, b, i, j - 1)));
    default: {
      const float2 dyym = hzd(eps_at(o, b, i - 1, j), eps_at(o, b, i - 2, j));
      const float2 dyyp = hzd(e, eps_at(o, b, i - 1, j));
      const float2 dxxm = hzd(eps_at(o, b, i, j - 1), eps_at(o, b, i, j - 2));
      const float2 dxxp = hzd(e, eps_at(o, b, i, j - 1));
      const float2 d0 = cadd(cadd(cmul(cx.am, dyym), cmul(cx.ap, dyyp)),
                             cadd(cmul(cy.am, dxxm), cmul(cy.ap, dxxp)));
      return csub(cscale(sh, k2), d0);
    }
  }
}

__device__ __forceinline__ float2 crcp(float2 d) {
  const float q = 1.0f / (d.x * d.x + d.y * d.y);
  return make_float2(d.x * q, -d.y * q);
}

// acc - c r in complex arithmetic, four FP32 FMAs in a fixed order.
__device__ __forceinline__ float2 cfms(float2 c, float2 r, float2 acc) {
  acc.x = fmaf(-c.x, r.x, acc.x);
  acc.x = fmaf(c.y, r.y, acc.x);
  acc.y = fmaf(-c.x, r.y, acc.y);
  acc.y = fmaf(-c.y, r.x, acc.y);
  return acc;
}

__device__ __forceinline__ void check_pivot(const Args& a, float2 d) {
  const float m = d.x * d.x + d.y * d.y;
  if (!(m > 0.f) || !isfinite(m)) atomicExch(a.fault, 1);
}

__device__ __forceinline__ float2* ftop(const Args& a, const Node& n, int b) {
  return a.fac + (long long)b * a.fac_pp + n.top;
}
__device__ __forceinline__ float2* fbl(const Args& a, const Node& n, int b) {
  return a.fac + (long long)b * a.fac_pp + n.bl;
}
__device__ __forceinline__ float2* fsch(const Args& a, const Node& n, int b) {
  return a.sar[n.par] + (long long)b * a.sa_pp[n.par] + n.s;
}
__device__ __forceinline__ float2* ffv(const Args& a, const Node& n, int b) {
  return a.fv + (long long)b * a.fv_pp + n.fv;
}

// Address of front entry (r, c) of a large node n for problem b.
__device__ __forceinline__ float2* fel(const Args& a, const Node& n, int b, int r, int c) {
  const int f = n.nI + n.nB;
  if (r < n.nI) return ftop(a, n, b) + (long long)r * f + c;
  r -= n.nI;
  if (c < n.nI) return fbl(a, n, b) + (long long)r * n.nI + c;
  return fsch(a, n, b) + (long long)r * n.nB + (c - n.nI);
}

// Zero [lo, lo + len) of every problem's block (stride pp elements).
__global__ void k_zero(float2* base, long long pp, long long lo, long long len, int B) {
  const long long total = len * B;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long b = e / len, k = e - b * len;
    base[b * pp + lo + k] = make_float2(0.f, 0.f);
  }
}

// ============================================================ small fronts
__device__ __forceinline__ float2 shfl2(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// Visits e = start, start + step, ... < total as (e, e / d, e % d) with one
// division up front instead of one per element.
template <typename Fn>
__device__ __forceinline__ void for_divmod(int start, int step, int total, int d, Fn&& fn) {
  int q = start / d, r = start - q * d;
  const int sq = step / d, sr = step - sq * d;
  for (int e = start; e < total; e += step) {
    fn(e, q, r);
    q += sq;
    r += sr;
    if (r >= d) {
      r -= d;
      ++q;
    }
  }
}

// Writes the swept front (row stride ld in shared memory) to the factor:
// [G | H] and -K column-major, S row-major.
__device__ __forceinline__ void store_small(const Args& a, const Node& n, int b, const float2* F,
                                            int ld, int tid, int nt) {
  const int nI = n.nI, nB = n.nB, f = nI + nB;
  float2* top = ftop(a, n, b);
  float2* bl = fbl(a, n, b);
  float2* S = fsch(a, n, b);
  for_divmod(tid, nt, nI * f, nI, [&](int e, int c, int r) { top[e] = F[r * ld + c]; });
  if (nB == 0) return;
  for_divmod(tid, nt, nB * nI, nB, [&](int e, int c, int r) { bl[e] = F[(nI + r) * ld + c]; });
  for_divmod(tid, nt, nB * nB, nB, [&](int e, int r, int c) { S[e] = F[(nI + r) * ld + nI + c]; });
}

// Leaves (childless fronts, nI <= 16, nB <= 16): F_BB = 0 and every boundary
// cell j couples to exactly one interior cell i_j, from one side (the frame of
// a box without its corners), so with G = F_II^-1 the sweep operator is
//   H[:, j] = G[:, i_j] a_j,   -K[j, :] = -b_j G[i_j, :],
//   S[j, l] = -b_j G[i_j, i_l] a_l,      a_j = F[i_j, j], b_j = F[j, i_j]:
// only the nI x nI inverse is computed.  One warp per (leaf, problem), no
// CTA barrier; G is swept pivot by pivot in registers (lane 2r + h holds
// columns 8h .. 8h + 7 of row r), the pivot row and column by shuffles, with
// partial pivoting: swapping two rows not yet swept swaps two equations, so
// the sweep yields (Pm F_II)^-1 = F_II^-1 Pm^T, whose columns are put back
// in order when G is stored.
constexpr int LEAF_WARPS = 4;
__global__ void __launch_bounds__(LEAF_WARPS * 32) k_leaf(Args a, const int* __restrict__ list,
                                                          int count) {
  __shared__ float2 Gs[LEAF_WARPS][16][17];
  __shared__ float2 av[LEAF_WARPS][16], bv[LEAF_WARPS][16];
  __shared__ int ia[LEAF_WARPS][16], ib[LEAF_WARPS][16];
  __shared__ int lperm[LEAF_WARPS][16];  // row i of the swept matrix is row lperm[i] of F_II
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * LEAF_WARPS + warp;
  if (item >= count) return;  // warp-uniform; the kernel has no CTA barrier
  const Node n = a.nodes[list[item]];
  const int b = blockIdx.y;
  const int nI = n.nI, nB = n.nB, f = nI + nB;
  float2(*G)[17] = Gs[warp];
  for (int e = lane; e < 256; e += 32) G[e >> 4][e & 15] = make_float2(0.f, 0.f);
  if (lane < 16) lperm[warp][lane] = lane;
  __syncwarp();
  for (int q = lane; q < n.ndesc; q += 32) {
    const Desc d = a.desc[n.desc + q];  // (row, col) pairs are distinct
    const float2 v = coef(a.op, b, d.cell, d.dir);
    if (d.row < nI) {
      if (d.col < nI) {
        G[d.row][d.col] = v;
      } else {
        av[warp][d.col - nI] = v;
        ia[warp][d.col - nI] = d.row;
      }
    } else {
      bv[warp][d.row - nI] = v;
      ib[warp][d.row - nI] = d.col;
    }
  }
  __syncwarp();
  const int r = lane >> 1, h = lane & 1;
  float2 x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = G[r][8 * h + k];
  for (int p = 0; p < nI; ++p) {
    // F[r, p] sits in lane 2r + p / 8, slot p % 8; F[p, 8h + k] in lane 2p + h, slot k
    float2 mine = x[0];
#pragma unroll
    for (int k = 1; k < 8; ++k)
      if ((p & 7) == k) mine = x[k];
    float2 colv = shfl2(mine, 2 * r + (p >> 3));
    // pivot row: the largest |F[q, p]| among rows p .. nI-1 (lowest row on ties)
    float m = (h == 0 && r >= p && r < nI) ? colv.x * colv.x + colv.y * colv.y : -1.f;
    int q = r;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float m2 = __shfl_xor_sync(0xffffffffu, m, o);
      const int q2 = __shfl_xor_sync(0xffffffffu, q, o);
      if (m2 > m || (m2 == m && q2 < q)) {
        m = m2;
        q = q2;
      }
    }
    if (q != p) {  // warp-uniform: rows p and q trade places
      const int src = r == p ? 2 * q + h : (r == q ? 2 * p + h : lane);
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = shfl2(x[k], src);
      colv = shfl2(colv, src);
      if (lane == 0) {
        const int t = lperm[warp][p];
        lperm[warp][p] = lperm[warp][q];
        lperm[warp][q] = t;
      }
    }
    const float2 piv = shfl2(colv, 2 * p);
    if (lane == 0) check_pivot(a, piv);
    const float2 pinv = crcp(piv);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int c = 8 * h + k;
      const float2 rv = shfl2(x[k], 2 * p + h);
      const float2 mult = c == p ? pinv : cmul(rv, pinv);
      const float2 base = c == p ? make_float2(0.f, 0.f) : x[k];
      x[k] = r == p ? mult : csub(base, cmul(colv, mult));
    }
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int c = 8 * h + k;
    G[r][c < nI ? lperm[warp][c] : c] = x[k];
  }
  __syncwarp();
  float2* top = ftop(a, n, b);
  for_divmod(lane, 32, nI * f, nI, [&](int e, int c, int rr) {
    top[e] = c < nI ? G[rr][c] : cmul(G[rr][ia[warp][c - nI]], av[warp][c - nI]);
  });
  if (nB == 0) return;
  float2* bl = fbl(a, n, b);
  float2* S = fsch(a, n, b);
  for_divmod(lane, 32, nB * nI, nB, [&](int e, int c, int j) {
    const float2 t = cmul(bv[warp][j], G[ib[warp][j]][c]);
    bl[e] = make_float2(-t.x, -t.y);
  });
  for_divmod(lane, 32, nB * nB, nB, [&](int e, int j, int l) {
    const float2 t = cmul(cmul(bv[warp][j], G[ib[warp][j]][ia[warp][l]]), av[warp][l]);
    S[e] = make_float2(-t.x, -t.y);
  });
}

// Other small fronts: one CTA of NT threads per (node, problem).  The front
// lives in shared memory (row stride ld, a multiple of 4 >= f, entries
// beyond f zero) and is swept in blocks P of up to BS pivots, each block in
// three phases:
//   A. warp 0: LU with partial (row) pivoting of F[P, P], Pm F[P, P] = L U,
//      padded with the identity to BS x BS; meanwhile the other warps copy the
//      old pivot columns F[r, P] (r outside P), transposed, to Ct.
//   B. row panel (a thread per column c): Rt[:, c] = L^-1 Pm F[P, c], then
//      F[P, c] = U^-1 Rt[:, c]; for c in P the right-hand side is the unit
//      vector, which writes F[P, P]^-1.  Column panel (a thread per row r):
//      Ct[:, r] = (F[r, P] U^-1)^T, then F[r, P] = -(Ct[:, r]^T L^-1) Pm.
// Only F[P, P]^-1 enters the sweep operator, so pivoting inside a block
// leaves the result unchanged and keeps small pivots of a near-resonant
// block from growing the rounding.
//   C. rank-|P| update F[r, c] -= Ct[:, r] . Rt[:, c] of the entries outside
//      the pivot rows and columns, a 4 x 4 register tile per thread and step.
// The pivot order is the same as a pivot-by-pivot Gauss-Jordan sweep, so the
// result is the same sweep operator.  The update takes the LU split
// (F_rP U^-1)(L^-1 F_Pc), the right-looking form: the product of the old
// column with the finished row panel, F_rP (A_PP^-1 F_Pc), is the same
// number mathematically but cancels an order of magnitude more rounding on
// ill-conditioned pivot blocks.  Three barriers per pivot block.
template <int NT, int BS>
__global__ void __launch_bounds__(NT, 768 / NT) k_front(Args a, const int* __restrict__ list, int ld) {
  static_assert(NT >= 64 && BS <= 32, "k_front shape");
  constexpr int NW = NT / 32;
  extern __shared__ __align__(16) float2 sm[];
  float2* F = sm;             // [ld][ld]
  float2* Ct = sm + ld * ld;  // [BS][ld]: pivot columns, transposed
  float2* Rt = Ct + BS * ld;  // [BS][ld]: L^-1 times the pivot rows
  __shared__ float2 LU[BS][BS + 1];
  __shared__ float2 dinv[BS];
  __shared__ int pv[BS];  // row k of Pm F[P, P] is row pv[k] of F[P, P]
  const Node n = a.nodes[list[blockIdx.x]];
  const int b = blockIdx.y;
  const int f = n.nI + n.nB, nI = n.nI;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  {
    float4* F4 = reinterpret_cast<float4*>(F);
    for (int e = tid; e < ld * ld / 2; e += NT) F4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  for (int q = tid; q < n.ndesc; q += NT) {
    const Desc d = a.desc[n.desc + q];
    const float2 v = coef(a.op, b, d.cell, d.dir);
    float2& t = F[d.row * ld + d.col];
    t = cadd(t, v);
  }
  __syncthreads();
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int ch = n.child[s];
    if (ch < 0) continue;
    const int cnB = a.nodes[ch].nB;
    const int* map = a.cmap + n.cmap[s];
    const float2* S = fsch(a, a.nodes[ch], b);
    for (int r = warp; r < cnB; r += NW) {
      float2* row = F + map[r] * ld;
      const float2* src = S + (size_t)r * cnB;
      for (int q = lane; q < cnB; q += 32) {
        float2& t = row[map[q]];
        t = cadd(t, src[q]);
      }
    }
    __syncthreads();
  }
  for (int k0 = 0; k0 < nI; k0 += BS) {
    const int nb = min(BS, nI - k0);
    auto inP = [&](int i) { return i >= k0 && i < k0 + nb; };
    // ---- A
    if (warp == 0) {
      if (lane < BS) {
#pragma unroll
        for (int r = 0; r < BS; ++r)
          LU[r][lane] = (r < nb && lane < nb) ? F[(k0 + r) * ld + k0 + lane]
                                              : make_float2(r == lane ? 1.f : 0.f, 0.f);
        pv[lane] = lane;
      }
      __syncwarp();
      for (int k = 0; k < BS; ++k) {
        if (k < nb) {
          // the largest |entry| of column k among rows k .. nb-1 (lowest row on ties)
          float m = -1.f;
          int q = k;
          if (lane >= k && lane < nb) {
            const float2 v = LU[lane][k];
            m = v.x * v.x + v.y * v.y;
            q = lane;
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            const float m2 = __shfl_xor_sync(0xffffffffu, m, o);
            const int q2 = __shfl_xor_sync(0xffffffffu, q, o);
            if (m2 > m || (m2 == m && q2 < q)) {
              m = m2;
              q = q2;
            }
          }
          if (q != k) {  // warp-uniform
            if (lane < BS) {
              const float2 t = LU[k][lane];
              LU[k][lane] = LU[q][lane];
              LU[q][lane] = t;
            }
            if (lane == 0) {
              const int t = pv[k];
              pv[k] = pv[q];
              pv[q] = t;
            }
          }
          __syncwarp();
        }
        const float2 piv = LU[k][k];
        if (k < nb && lane == 0) check_pivot(a, piv);
        const float2 pinv = crcp(piv);
        if (lane > k && lane < BS) LU[lane][k] = cmul(LU[lane][k], pinv);
        __syncwarp();
        if (lane > k && lane < BS) {
          const float2 ukj = LU[k][lane];
#pragma unroll
          for (int r = 1; r < BS; ++r)
            if (r > k) LU[r][lane] = csub(LU[r][lane], cmul(LU[r][k], ukj));
        }
        __syncwarp();
      }
      if (lane < BS) dinv[lane] = crcp(LU[lane][lane]);
    } else {
      for (int k = warp - 1; k < BS; k += NW - 1)
        for (int r = lane; r < ld; r += 32)
          Ct[k * ld + r] = (k < nb && r < f && !inP(r)) ? F[r * ld + k0 + k] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    // ---- B (NT / 2 >= ld threads per panel)
    if (tid < NT / 2) {
      const int c = tid;
      if (c < f) {
        const bool piv = inP(c);
        float2 x[BS];
#pragma unroll
        for (int r = 0; r < BS; ++r)
          x[r] = piv ? make_float2(pv[r] == c - k0 ? 1.f : 0.f, 0.f)
                     : (r < nb ? F[(k0 + pv[r]) * ld + c] : make_float2(0.f, 0.f));
#pragma unroll
        for (int r = 1; r < BS; ++r)
#pragma unroll
          for (int k = 0; k < r; ++k) x[r] = csub(x[r], cmul(LU[r][k], x[k]));
#pragma unroll
        for (int r = 0; r < BS; ++r) Rt[r * ld + c] = x[r];
#pragma unroll
        for (int r = BS - 1; r >= 0; --r) {
#pragma unroll
          for (int k = r + 1; k < BS; ++k) x[r] = csub(x[r], cmul(LU[r][k], x[k]));
          x[r] = cmul(x[r], dinv[r]);
        }
#pragma unroll
        for (int r = 0; r < BS; ++r)
          if (r < nb) F[(k0 + r) * ld + c] = x[r];
      } else if (c < ld) {
#pragma unroll
        for (int r = 0; r < BS; ++r) Rt[r * ld + c] = make_float2(0.f, 0.f);
      }
    } else {
      const int r = tid - NT / 2;
      if (r < f && !inP(r)) {
        float2 x[BS];
#pragma unroll
        for (int k = 0; k < BS; ++k) x[k] = Ct[k * ld + r];
        // x U = a (left to right), then x L = y (right to left)
#pragma unroll
        for (int j = 0; j < BS; ++j) {
#pragma unroll
          for (int k = 0; k < j; ++k) x[j] = csub(x[j], cmul(x[k], LU[k][j]));
          x[j] = cmul(x[j], dinv[j]);
        }
#pragma unroll
        for (int k = 0; k < BS; ++k) Ct[k * ld + r] = x[k];
#pragma unroll
        for (int j = BS - 2; j >= 0; --j)
#pragma unroll
          for (int k = j + 1; k < BS; ++k) x[j] = csub(x[j], cmul(x[k], LU[k][j]));
#pragma unroll
        for (int k = 0; k < BS; ++k)
          if (k < nb) F[r * ld + k0 + pv[k]] = make_float2(-x[k].x, -x[k].y);
      }
    }
    __syncthreads();
    // ---- C
    {
      const int tcn = ld >> 2;
      for_divmod(tid, NT, tcn * tcn, tcn, [&](int, int tr, int tc) {
        const int R0 = tr * 4, C0 = tc * 4;
        if ((R0 >= k0 && R0 + 4 <= k0 + nb) || (C0 >= k0 && C0 + 4 <= k0 + nb)) return;
        float2 acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 u = *reinterpret_cast<const float4*>(F + (R0 + i) * ld + C0);
          const float4 w = *reinterpret_cast<const float4*>(F + (R0 + i) * ld + C0 + 2);
          acc[i][0] = make_float2(u.x, u.y);
          acc[i][1] = make_float2(u.z, u.w);
          acc[i][2] = make_float2(w.x, w.y);
          acc[i][3] = make_float2(w.z, w.w);
        }
#pragma unroll 4
        for (int k = 0; k < nb; ++k) {
          const float4 c01 = *reinterpret_cast<const float4*>(Ct + k * ld + R0);
          const float4 c23 = *reinterpret_cast<const float4*>(Ct + k * ld + R0 + 2);
          const float4 r01 = *reinterpret_cast<const float4*>(Rt + k * ld + C0);
          const float4 r23 = *reinterpret_cast<const float4*>(Rt + k * ld + C0 + 2);
          const float2 cv[4] = {make_float2(c01.x, c01.y), make_float2(c01.z, c01.w),
                                make_float2(c23.x, c23.y), make_float2(c23.z, c23.w)};
          const float2 rv[4] = {make_float2(r01.x, r01.y), make_float2(r01.z, r01.w),
                                make_float2(r23.x, r23.y), make_float2(r23.z, r23.w)};
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = cfms(cv[i], rv[j], acc[i][j]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          if (inP(R0 + i)) continue;
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (!inP(C0 + j)) F[(R0 + i) * ld + C0 + j] = acc[i][j];
        }
      });
    }
    __syncthreads();
  }
  store_small(a, n, b, F, ld, tid, NT);
}

// ============================================================ large fronts
// Original entries of the large fronts (fronts zeroed beforehand).
__global__ void k_orig(Args a, const int* __restrict__ list) {
  const Node n = a.nodes[list[blockIdx.x]];
  const int b = blockIdx.y;
  for (int q = threadIdx.x; q < n.ndesc; q += blockDim.x) {
    const Desc d = a.desc[n.desc + q];
    float2* t = fel(a, n, b, d.row, d.col);
    *t = cadd(*t, coef(a.op, b, d.cell, d.dir));
  }
}

// Extend-add of one child's Schur complement, one child row per CTA
// (work: node index, child row).
__global__ void k_extend(Args a, const int2* __restrict__ work, int slot) {
  const int2 w = work[blockIdx.x];
  const Node n = a.nodes[w.x];
  const int b = blockIdx.y;
  const int ch = slot == 0 ? n.child[0] : n.child[1];
  const int cm = slot == 0 ? n.cmap[0] : n.cmap[1];
  const Node c = a.nodes[ch];
  const int* map = a.cmap + cm;
  const int r = w.y;
  const float2* S = fsch(a, c, b) + (long long)r * c.nB;
  const int pr = map[r];
  for (int q = threadIdx.x; q < c.nB; q += blockDim.x) {
    float2* t = fel(a, n, b, pr, map[q]);
    *t = cadd(*t, S[q]);
  }
}

// Block step of a large front over the pivots P = [k0, k0 + nb), nb <= NB,
// in four launches:
//   k_pivblock: LU with partial (row) pivoting, Pm A_pp = L U (padded with
//     the identity to NB x NB), to the scratch `lub` / `lpv`, and
//     A_pp^-1 = U^-1 L^-1 Pm over A_pp in the front;
//   k_rowpanel: RB = L^-1 Pm F[P, c] (scratch) and F[P, c] = U^-1 RB for the
//     columns outside P;
//   k_colpanel: CB = F[r, P] U^-1 (scratch) and F[r, P] = -(CB L^-1) Pm for
//     the rows outside P;
//   k_update: F[r, c] -= CB[r, :] RB[:, c] outside the pivot rows and columns.
// The update takes the LU split (F_rP U^-1)(L^-1 Pm F_Pc), the right-looking
// form; the product of the old column with the finished row panel,
// F_rP (A_pp^-1 F_Pc), is the same number but cancels more rounding on
// ill-conditioned pivot blocks, and explicit-inverse panels lose about two
// orders of magnitude on Helmholtz fronts in complex64.  Pivoting inside the
// block leaves the sweep operator unchanged (only A_pp^-1 enters it).
__device__ __forceinline__ float2* lub_of(const Args& a, const Node& n, int b, int count) {
  return a.lub + ((size_t)b * count + n.lidx) * NB * NB;
}
__device__ __forceinline__ int* lpv_of(const Args& a, const Node& n, int b, int count) {
  return a.lpv + ((size_t)b * count + n.lidx) * NB;
}
__device__ __forceinline__ float2* rb_of(const Args& a, const Node& n, int b) {  // [NB][f]
  return a.rb + (size_t)b * a.ps_pp + (size_t)n.po * NB;
}
__device__ __forceinline__ float2* cb_of(const Args& a, const Node& n, int b) {  // [f][NB]
  return a.cb + (size_t)b * a.ps_pp + (size_t)n.po * NB;
}

// One warp per (large front, problem).
__global__ void __launch_bounds__(128) k_pivblock(Args a, const int* __restrict__ list, int count,
                                                  int k0) {
  __shared__ float2 blk[4][NB][NB + 1];
  __shared__ int pvs[4][NB];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * 4 + warp;
  if (item >= count) return;
  const Node n = a.nodes[list[item]];
  if (k0 >= n.nI) return;
  const int b = blockIdx.y;
  const int nb = min(NB, n.nI - k0), f = n.nI + n.nB;
  float2* base = ftop(a, n, b);
  float2(*B)[NB + 1] = blk[warp];
  int* pv = pvs[warp];
  for (int r = 0; r < NB; ++r)
    B[r][lane] = (r < nb && lane < nb) ? base[(size_t)(k0 + r) * f + k0 + lane]
                                       : make_float2(r == lane ? 1.f : 0.f, 0.f);
  pv[lane] = lane;
  __syncwarp();
  // LU with partial pivoting, lane j owns column j
  for (int k = 0; k < NB; ++k) {
    if (k < nb) {
      float m = -1.f;
      int q = k;
      if (lane >= k && lane < nb) {
        const float2 v = B[lane][k];
        m = v.x * v.x + v.y * v.y;
        q = lane;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float m2 = __shfl_xor_sync(0xffffffffu, m, o);
        const int q2 = __shfl_xor_sync(0xffffffffu, q, o);
        if (m2 > m || (m2 == m && q2 < q)) {
          m = m2;
          q = q2;
        }
      }
      if (q != k) {  // warp-uniform
        const float2 t = B[k][lane];
        B[k][lane] = B[q][lane];
        B[q][lane] = t;
        if (lane == 0) {
          const int ti = pv[k];
          pv[k] = pv[q];
          pv[q] = ti;
        }
      }
      __syncwarp();
    }
    const float2 piv = B[k][k];
    if (k < nb && lane == 0) check_pivot(a, piv);
    const float2 pinv = crcp(piv);
    if (lane > k) B[lane][k] = cmul(B[lane][k], pinv);
    __syncwarp();
    if (lane > k) {
      const float2 ukj = B[k][lane];
      for (int r = k + 1; r < NB; ++r) B[r][lane] = csub(B[r][lane], cmul(B[r][k], ukj));
    }
    __syncwarp();
  }
  float2* lu = lub_of(a, n, b, count);
  for (int r = 0; r < NB; ++r) lu[r * NB + lane] = B[r][lane];
  lpv_of(a, n, b, count)[lane] = pv[lane];
  // column `lane` of A_pp^-1 = U^-1 L^-1 Pm e_lane
  float2 y[NB];
#pragma unroll
  for (int r = 0; r < NB; ++r) {
    float2 t = make_float2(pv[r] == lane ? 1.f : 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < r; ++k) t = csub(t, cmul(B[r][k], y[k]));
    y[r] = t;
  }
#pragma unroll
  for (int r = NB - 1; r >= 0; --r) {
    float2 t = y[r];
#pragma unroll
    for (int k = r + 1; k < NB; ++k) t = csub(t, cmul(B[r][k], y[k]));
    y[r] = cmul(t, crcp(B[r][r]));
  }
  if (lane < nb)
#pragma unroll
    for (int r = 0; r < NB; ++r)
      if (r < nb) base[(size_t)(k0 + r) * f + k0 + lane] = y[r];
}

// Pivot rows, one thread per column (work: node index, column chunk of TILE).
__global__ void __launch_bounds__(TILE) k_rowpanel(Args a, const int2* __restrict__ work, int k0,
                                                   int count) {
  __shared__ float2 LU[NB][NB + 1];
  __shared__ float2 dinv[NB];
  __shared__ int pv[NB];
  const int2 w = work[blockIdx.x];
  const Node n = a.nodes[w.x];
  if (k0 >= n.nI) return;
  const int b = blockIdx.y;
  const int nb = min(NB, n.nI - k0), f = n.nI + n.nB;
  const float2* lu = lub_of(a, n, b, count);
  for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) LU[e / NB][e % NB] = lu[e];
  if (threadIdx.x < NB) pv[threadIdx.x] = lpv_of(a, n, b, count)[threadIdx.x];
  __syncthreads();
  if (threadIdx.x < NB) dinv[threadIdx.x] = crcp(LU[threadIdx.x][threadIdx.x]);
  __syncthreads();
  const int c = w.y * TILE + threadIdx.x;
  if (c >= f) return;
  float2* rb = rb_of(a, n, b);
  if (c >= k0 && c < k0 + nb) {  // the pivot block's columns carry nothing into the update
#pragma unroll
    for (int r = 0; r < NB; ++r) rb[(size_t)r * f + c] = make_float2(0.f, 0.f);
    return;
  }
  float2* base = ftop(a, n, b);
  float2 x[NB];
#pragma unroll
  for (int r = 0; r < NB; ++r)
    x[r] = r < nb ? base[(size_t)(k0 + pv[r]) * f + c] : make_float2(0.f, 0.f);
#pragma unroll
  for (int r = 1; r < NB; ++r)
#pragma unroll
    for (int k = 0; k < r; ++k) x[r] = csub(x[r], cmul(LU[r][k], x[k]));
#pragma unroll
  for (int r = 0; r < NB; ++r) rb[(size_t)r * f + c] = x[r];
#pragma unroll
  for (int r = NB - 1; r >= 0; --r) {
#pragma unroll
    for (int k = r + 1; k < NB; ++k) x[r] = csub(x[r], cmul(LU[r][k], x[k]));
    x[r] = cmul(x[r], dinv[r]);
  }
#pragma unroll
  for (int r = 0; r < NB; ++r)
    if (r < nb) base[(size_t)(k0 + r) * f + c] = x[r];
}

// Pivot columns, one thread per row (work: node index, row chunk of TILE).
__global__ void __launch_bounds__(TILE) k_colpanel(Args a, const int2* __restrict__ work, int k0,
                                                   int count) {
  __shared__ float2 LU[NB][NB + 1];
  __shared__ float2 dinv[NB];
  __shared__ int pv[NB];
  __shared__ float2 P[TILE][NB + 1];
  const int2 w = work[blockIdx.x];
  const Node n = a.nodes[w.x];
  if (k0 >= n.nI) return;
  const int b = blockIdx.y;
  const int nb = min(NB, n.nI - k0), f = n.nI + n.nB;
  const int r0 = w.y * TILE;
  const float2* lu = lub_of(a, n, b, count);
  for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) LU[e / NB][e % NB] = lu[e];
  if (threadIdx.x < NB) pv[threadIdx.x] = lpv_of(a, n, b, count)[threadIdx.x];
  for (int e = threadIdx.x; e < TILE * NB; e += blockDim.x) {
    const int i = e / NB, k = e - i * NB;
    const int r = r0 + i;
    P[i][k] = (r < f && k < nb) ? *fel(a, n, b, r, k0 + k) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  if (threadIdx.x < NB) dinv[threadIdx.x] = crcp(LU[threadIdx.x][threadIdx.x]);
  __syncthreads();
  float2* cb = cb_of(a, n, b);
  const int i = threadIdx.x, r = r0 + i;
  if (r < f && !(r >= k0 && r < k0 + nb)) {
    float2 x[NB];
#pragma unroll
    for (int k = 0; k < NB; ++k) x[k] = P[i][k];
    // x U = a (columns left to right): the update's left factor
#pragma unroll
    for (int j = 0; j < NB; ++j) {
#pragma unroll
      for (int k = 0; k < j; ++k) x[j] = csub(x[j], cmul(x[k], LU[k][j]));
      x[j] = cmul(x[j], dinv[j]);
    }
#pragma unroll
    for (int k = 0; k < NB; ++k) cb[(size_t)r * NB + k] = x[k];
    // then x L = y (right to left); column k of the result belongs to pivot pv[k]
#pragma unroll
    for (int j = NB - 2; j >= 0; --j)
#pragma unroll
      for (int k = j + 1; k < NB; ++k) x[j] = csub(x[j], cmul(x[k], LU[k][j]));
#pragma unroll
    for (int k = 0; k < NB; ++k) P[i][k] = make_float2(-x[k].x, -x[k].y);
  } else if (r < f) {
#pragma unroll
    for (int k = 0; k < NB; ++k) cb[(size_t)r * NB + k] = make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < TILE * NB; e += blockDim.x) {
    const int ii = e / NB, k = e - ii * NB;
    const int rr = r0 + ii;
    if (k >= nb || rr >= f || (rr >= k0 && rr < k0 + nb)) continue;
    *fel(a, n, b, rr, k0 + pv[k]) = P[ii][k];
  }
}

// Rank-nb update of every entry outside the pivot rows and columns:
// F[r, c] -= CB[r, :] RB[:, c], one UT_R x UT_C tile per CTA (work: node,
// tile).  128 threads, each an 8 x 4 block (rows ty + 8u, cols tx + 16v);
// four CTAs per SM, so one CTA's loads overlap another's FMAs.  Each
// accumulator starts from the entry's old value, loaded before the panels,
// so the read-modify-write latency overlaps the panel loads.
constexpr int UT_R = 64, UT_C = 64, UT_NT = 128;
constexpr int UPD_SMEM = (UT_R * (NB + 1) + NB * UT_C) * (int)sizeof(float2);

__global__ void __launch_bounds__(UT_NT, 4) k_update(Args a, const int2* __restrict__ work, int k0) {
  extern __shared__ float2 usm[];
  float2(*Cp)[NB + 1] = (float2(*)[NB + 1])usm;                  // [UT_R][NB + 1]
  float2(*Rp)[UT_C] = (float2(*)[UT_C])(usm + UT_R * (NB + 1));  // [NB][UT_C]
  const int2 w = work[blockIdx.x];
  const Node n = a.nodes[w.x];
  if (k0 >= n.nI) return;
  const int b = blockIdx.y;
  const int nI = n.nI, nB = n.nB;
  const int nb = min(NB, nI - k0), f = nI + nB;
  const int tc = (f + UT_C - 1) / UT_C;
  const int r0 = (w.y / tc) * UT_R, c0 = (w.y % tc) * UT_C;
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;  // ty < 8
  float2* const top = ftop(a, n, b);
  float2* const bl = fbl(a, n, b);
  float2* const sch = fsch(a, n, b);
  // row r of the front: entries c < nI at lo[c], entries c >= nI at hi[c]
  auto row_lo = [&](int r) { return r < nI ? top + (size_t)r * f : bl + (size_t)(r - nI) * nI; };
  auto row_hi = [&](int r) {
    return r < nI ? top + (size_t)r * f : sch + (size_t)(r - nI) * nB - nI;
  };
  // old values of this thread's entries (0 where outside or in the pivot block)
  float2 acc[8][4];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int r = r0 + ty + 8 * u;
    const bool rok = r < f && !(r >= k0 && r < k0 + nb);
    const float2* lo = row_lo(min(r, f - 1));
    const float2* hi = row_hi(min(r, f - 1));
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = c0 + tx + 16 * v;
      acc[u][v] = (rok && c < f && !(c >= k0 && c < k0 + nb)) ? (c < nI ? lo[c] : hi[c])
                                                               : make_float2(0.f, 0.f);
    }
  }
  // panels: CB rows r0 .. r0 + UT_R - 1, RB columns c0 .. c0 + UT_C - 1
  {
    const float2* cb = cb_of(a, n, b);
    const int k = threadIdx.x & (NB - 1);
#pragma unroll 4
    for (int i = threadIdx.x >> 5; i < UT_R; i += UT_NT / 32) {
      const int r = r0 + i;
      Cp[i][k] = (r < f && k < nb) ? cb[(size_t)r * NB + k] : make_float2(0.f, 0.f);
    }
  }
  {
    const float2* rb = rb_of(a, n, b);
    const int j = threadIdx.x & (UT_C - 1);
    const int c = c0 + j;
#pragma unroll 4
    for (int k = threadIdx.x >> 6; k < NB; k += UT_NT / 64)
      Rp[k][j] = (k < nb && c < f) ? rb[(size_t)k * f + c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
#pragma unroll 4
  for (int k = 0; k < NB; ++k) {
    float2 cv[8], rv[4];
#pragma unroll
    for (int u = 0; u < 8; ++u) cv[u] = Cp[ty + 8 * u][k];
#pragma unroll
    for (int v = 0; v < 4; ++v) rv[v] = Rp[k][tx + 16 * v];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = cfms(cv[u], rv[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int r = r0 + ty + 8 * u;
    if (r >= f || (r >= k0 && r < k0 + nb)) continue;
    float2* lo = row_lo(r);
    float2* hi = row_hi(r);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = c0 + tx + 16 * v;
      if (c >= f || (c >= k0 && c < k0 + nb)) continue;
      (c < nI ? lo : hi)[c] = acc[u][v];
    }
  }
}

// ================================================================ apply
struct ApplyIO {
  const float2* v;   // [B][n] input (Krylov basis vector)
  float2* z;         // [B][n] output
  const double* sc;  // per-problem input scale sc[b * sc_stride + sc_index] (NULL: 1)
  int sc_stride, sc_index;
  const KState* st;  // skip problems whose Arnoldi work is off (NULL: none)
};

__device__ __forceinline__ bool skip(const ApplyIO& io, int b) {
  return io.st != nullptr && !io.st[b].active;
}

__device__ __forceinline__ float in_scale(const ApplyIO& io, int b) {
  return io.sc ? (float)io.sc[(size_t)b * io.sc_stride + io.sc_index] : 1.f;
}

// Front vector f = [s v_I ; 0] + the children's update vectors, in fvs
// (lanes or threads stride by `step`); callers sync before reading it.
__device__ __forceinline__ void gather_front(const Args& a, const ApplyIO& io, const Node& n, int b,
                                             float2* fvs, int t0, int step, bool warp_only) {
  const int f = n.nI + n.nB;
  const float s = in_scale(io, b);
  const int* cl = a.cells + n.cells;
  const float2* v = io.v + (size_t)b * a.n;
  for (int t = t0; t < f; t += step) fvs[t] = t < n.nI ? cscale(v[cl[t]], s) : make_float2(0.f, 0.f);
  if (warp_only) __syncwarp(); else __syncthreads();
#pragma unroll
  for (int sl = 0; sl < 2; ++sl) {
    const int ch = n.child[sl];
    if (ch < 0) continue;
    const Node c = a.nodes[ch];
    const int* map = a.cmap + n.cmap[sl];
    const float2* u = ffv(a, c, b) + c.nI;
    for (int t = t0; t < c.nB; t += step) {
      float2& d = fvs[map[t]];
      d = cadd(d, u[t]);
    }
    if (warp_only) __syncwarp(); else __syncthreads();
  }
}

// y[r] = sum_k M[k * rows + r] x[k] for r < rows (column-major M in global
// memory, x in shared memory), one warp; returns y[r] in the lanes with
// lane % 32 == r (32-row chunks, call per chunk).  With rows <= 16 the two
// half-warps take alternate k and are added by a shuffle; each lane keeps 8
// independent loads in flight.
__device__ __forceinline__ float2 colmajor_gemv(const float2* __restrict__ M, const float2* x,
                                                int rows, int cols, int r0, int lane) {
  const int g = rows - r0 <= 16 ? 2 : 1;
  const int r = r0 + (g == 2 ? (lane & 15) : lane);
  const int k0 = g == 2 ? (lane >> 4) : 0;
  float2 a0 = make_float2(0.f, 0.f), a1 = a0;
  if (r < rows) {
    int k = k0;
    for (; k + 7 * g < cols; k += 8 * g) {
      float2 t[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) t[j] = __ldg(M + (size_t)(k + j * g) * rows + r);
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        a0 = cfma(t[j], x[k + j * g], a0);
        a1 = cfma(t[j + 1], x[k + (j + 1) * g], a1);
      }
    }
    for (; k < cols; k += g) a0 = cfma(__ldg(M + (size_t)k * rows + r), x[k], a0);
  }
  float2 acc = cadd(a0, a1);
  if (g == 2) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 16);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 16);
  }
  return acc;
}

// Forward, small fronts: one warp per (front, problem):
// u = f_B + (-K) f_I from the column-major -K.
__global__ void __launch_bounds__(WPB * 32) k_fwd_small(Args a, ApplyIO io,
                                                        const int* __restrict__ list, int count) {
  __shared__ float2 buf[WPB][SMALL_F];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * WPB + warp;
  const int b = blockIdx.y;
  if (item >= count || skip(io, b)) return;
  const Node n = a.nodes[list[item]];
  float2* fvs = buf[warp];
  gather_front(a, io, n, b, fvs, lane, 32, true);
  const float2* K = fbl(a, n, b);
  float2* out = ffv(a, n, b);
  for (int r0 = 0; r0 < n.nB; r0 += 32) {
    const float2 acc = colmajor_gemv(K, fvs, n.nB, n.nI, r0, lane);
    const int r = r0 + lane;
    if (r < n.nB && (n.nB - r0 > 16 || lane < 16)) out[n.nI + r] = cadd(fvs[n.nI + r], acc);
  }
  for (int t = lane; t < n.nI; t += 32) out[t] = fvs[t];
}

// Backward, small fronts: one warp per (front, problem):
// x_I = [G | H] w, w = [f_I ; -x_B], from the column-major factor.
__global__ void __launch_bounds__(WPB * 32) k_bwd_small(Args a, ApplyIO io,
                                                        const int* __restrict__ list, int count) {
  __shared__ float2 buf[WPB][SMALL_F];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int item = blockIdx.x * WPB + warp;
  const int b = blockIdx.y;
  if (item >= count || skip(io, b)) return;
  const Node n = a.nodes[list[item]];
  const int f = n.nI + n.nB;
  float2* wv = buf[warp];
  const float2* fvn = ffv(a, n, b);
  const int* cl = a.cells + n.cells;
  float2* z = io.z + (size_t)b * a.n;
  for (int t = lane; t < f; t += 32) {
    if (t < n.nI) {
      wv[t] = fvn[t];
    } else {
      const float2 x = z[cl[t]];
      wv[t] = make_float2(-x.x, -x.y);
    }
  }
  __syncwarp();
  const float2* T = ftop(a, n, b);
  for (int r0 = 0; r0 < n.nI; r0 += 32) {
    const float2 acc = colmajor_gemv(T, wv, n.nI, f, r0, lane);
    const int r = r0 + lane;
    if (r < n.nI && (n.nI - r0 > 16 || lane < 16)) z[cl[r]] = acc;
  }
}

// Forward gather of a large front (one CTA per front and problem).
__global__ void __launch_bounds__(256) k_fwd_large(Args a, ApplyIO io, const int* __restrict__ list) {
  extern __shared__ float2 fvs[];
  const Node n = a.nodes[list[blockIdx.x]];
  const int b = blockIdx.y;
  if (skip(io, b)) return;
  gather_front(a, io, n, b, fvs, threadIdx.x, blockDim.x, false);
  float2* out = ffv(a, n, b);
  for (int t = threadIdx.x; t < n.nI + n.nB; t += blockDim.x) out[t] = fvs[t];
}

// Row dot product of a warp: sum_k row[k] x[k]; each lane keeps 8
// independent loads in flight (four partial sums).
__device__ __forceinline__ float2 warp_dot(const float2* __restrict__ row, const float2* x, int len,
                                           int lane) {
  float2 a0 = make_float2(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
  int k = lane;
  for (; k + 224 < len; k += 256) {
    float2 t[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) t[j] = __ldg(row + k + 32 * j);
    a0 = cfma(t[0], x[k], a0);
    a1 = cfma(t[1], x[k + 32], a1);
    a2 = cfma(t[2], x[k + 64], a2);
    a3 = cfma(t[3], x[k + 96], a3);
    a0 = cfma(t[4], x[k + 128], a0);
    a1 = cfma(t[5], x[k + 160], a1);
    a2 = cfma(t[6], x[k + 192], a2);
    a3 = cfma(t[7], x[k + 224], a3);
  }
  for (; k < len; k += 32) a0 = cfma(__ldg(row + k), x[k], a0);
  float2 acc = cadd(cadd(a0, a1), cadd(a2, a3));
  acc.x = warp_sumf(acc.x);
  acc.y = warp_sumf(acc.y);
  return acc;
}

// Forward GEMV of a large front: u[r] += (-K)[r] f_I for GEMV_ROWS rows
// (work: node, row chunk).
__global__ void __launch_bounds__(256) k_fwd_gemv(Args a, ApplyIO io, const int2* __restrict__ work) {
  extern __shared__ float2 fi[];
  const int2 w = work[blockIdx.x];
  const Node n = a.nodes[w.x];
  const int b = blockIdx.y;
  if (skip(io, b)) return;
  float2* fvn = ffv(a, n, b);
  for (int t = threadIdx.x; t < n.nI; t += blockDim.x) fi[t] = fvn[t];
  __syncthreads();
  const float2* K = fbl(a, n, b);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int r1 = min(n.nB, (w.y + 1) * GEMV_ROWS);
  for (int r = w.y * GEMV_ROWS + warp; r < r1; r += nw) {
    const float2 acc = warp_dot(K + (size_t)r * n.nI, fi, n.nI, lane);
    if (lane == 0) fvn[n.nI + r] = cadd(fvn[n.nI + r], acc);
  }
}

// Backward of a large front: x_I = [G | H] [f_I ; -x_B] for GEMV_ROWS rows
// (work: node, row chunk).
__global__ void __launch_bounds__(256) k_bwd_large(Args a, ApplyIO io, const int2* __restrict__ work) {
  extern __shared__ float2 wv[];
  const int2 w = work[blockIdx.x];
  const Node n = a.nodes[w.x];
  const int b = blockIdx.y;
  if (skip(io, b)) return;
  const int f = n.nI + n.nB;
  const float2* fvn = ffv(a, n, b);
  const int* cl = a.cells + n.cells;
  float2* z = io.z + (size_t)b * a.n;
  for (int t = threadIdx.x; t < f; t += blockDim.x) {
    if (t < n.nI) {
      wv[t] = fvn[t];
    } else {
      const float2 x = z[cl[t]];
      wv[t] = make_float2(-x.x, -x.y);
    }
  }
  __syncthreads();
  const float2* T = ftop(a, n, b);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int r1 = min(n.nI, (w.y + 1) * GEMV_ROWS);
  for (int r = w.y * GEMV_ROWS + warp; r < r1; r += nw) {
    const float2 acc = warp_dot(T + (size_t)r * f, wv, f, lane);
    if (lane == 0) z[cl[r]] = acc;
  }
}

// ============================================================ host side
struct HNode {
  int x0, x1, y0, y1, depth;
  int child[2] = {-1, -1};
  std::vector<int> I, B;
};

static void build_tree(std::vector<HNode>& nodes, int nx, int ny, int x0, int x1, int y0, int y1,
                       int depth) {
  // explicit stack: (box, depth, parent, child slot)
  struct Item {
    int x0, x1, y0, y1, depth, parent, slot;
  };
  std::vector<Item> stack{{x0, x1, y0, y1, depth, -1, 0}};
  while (!stack.empty()) {
    const Item it = stack.back();
    stack.pop_back();
    if (it.x1 <= it.x0 || it.y1 <= it.y0) continue;
    const int id = (int)nodes.size();
    nodes.push_back(HNode());
    HNode& h = nodes.back();
    h.x0 = it.x0; h.x1 = it.x1; h.y0 = it.y0; h.y1 = it.y1; h.depth = it.depth;
    if (it.parent >= 0) {
      HNode& p = nodes[it.parent];
      if (p.child[0] < 0) p.child[0] = id; else p.child[1] = id;
    }
    const int w = it.x1 - it.x0, hh = it.y1 - it.y0;
    HNode& g = nodes[id];
    if (w <= LEAF && hh <= LEAF) {
      for (int i = it.x0; i < it.x1; ++i)
        for (int j = it.y0; j < it.y1; ++j) g.I.push_back(i * ny + j);
    } else if (w >= hh) {
      const int xs = it.x0 + w / 2;
      for (int j = it.y0; j < it.y1; ++j) g.I.push_back(xs * ny + j);
      stack.push_back({xs + 1, it.x1, it.y0, it.y1, it.depth + 1, id, 1});
      stack.push_back({it.x0, xs, it.y0, it.y1, it.depth + 1, id, 0});
    } else {
      const int ys = it.y0 + hh / 2;
      for (int i = it.x0; i < it.x1; ++i) g.I.push_back(i * ny + ys);
      stack.push_back({it.x0, it.x1, ys + 1, it.y1, it.depth + 1, id, 1});
      stack.push_back({it.x0, it.x1, it.y0, ys, it.depth + 1, id, 0});
    }
    if (it.x0 > 0) for (int j = it.y0; j < it.y1; ++j) g.B.push_back((it.x0 - 1) * ny + j);
    if (it.x1 < nx) for (int j = it.y0; j < it.y1; ++j) g.B.push_back(it.x1 * ny + j);
    if (it.y0 > 0) for (int i = it.x0; i < it.x1; ++i) g.B.push_back(i * ny + it.y0 - 1);
    if (it.y1 < ny) for (int i = it.x0; i < it.x1; ++i) g.B.push_back(i * ny + it.y1);
  }
}

struct Level {
  std::vector<int> small, large;            // node ids
  std::vector<int> leaf, front;             // small fronts: leaves (k_leaf), the rest (k_front)
  std::vector<int2> ext[2], panel, tiles;   // large-front work lists
  std::vector<int2> gemv, bwd;              // large-front apply work lists
  int max_f_small = 0, max_nI_small = 0, max_f_large = 0, max_nI_large = 0;
  long long fac_lo = 0, fac_len = 0, s_len = 0;  // per-problem ranges of this depth
  int *d_small = nullptr, *d_large = nullptr, *d_leaf = nullptr, *d_front = nullptr;
  int2 *d_ext[2] = {nullptr, nullptr}, *d_panel = nullptr, *d_tiles = nullptr;
  int2 *d_gemv = nullptr, *d_bwd = nullptr;
};

// Symbolic part of the factorisation: depends on the grid only, shared by
// every handle of that grid on a device.
struct Shape {
  int nx = 0, ny = 0, device = -1, ndepth = 0;
  std::vector<Level> levels;
  Node* d_nodes = nullptr;
  int* d_cells = nullptr;
  int* d_cmap = nullptr;
  Desc* d_desc = nullptr;
  long long fac_pp = 0, sa_pp[2] = {0, 0}, fv_pp = 0;
  long long ps_pp = 0;  // panel scratch per problem: NB x (sum of f over a depth's large fronts)
  double cmacs_pp = 0;  // Gauss-Jordan complex multiply-adds per problem
  size_t n_nodes = 0, n_desc = 0;
  long long cover[2] = {0, 0};
  ~Shape() {
    if (device < 0) return;  // host-only analysis: nothing on a device
    for (auto& L : levels) {
      cudaFree(L.d_small); cudaFree(L.d_large); cudaFree(L.d_leaf); cudaFree(L.d_front);
      cudaFree(L.d_ext[0]); cudaFree(L.d_ext[1]);
      cudaFree(L.d_panel); cudaFree(L.d_tiles); cudaFree(L.d_gemv); cudaFree(L.d_bwd);
    }
    cudaFree(d_nodes); cudaFree(d_cells); cudaFree(d_cmap); cudaFree(d_desc);
  }
};

template <typename T>
static int upload(T** dst, const std::vector<T>& v) {
  *dst = nullptr;
  if (v.empty()) return CEV_OK;
  CEV_CUDA(cudaMalloc((void**)dst, sizeof(T) * v.size()));
  CEV_CUDA(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return CEV_OK;
}

// A front k_leaf can sweep: no children, nI and nB <= 16, and each boundary
// cell coupled to exactly one interior cell in each direction (one F_IB entry
// in its column, one F_BI entry in its row) -- the leaves of the dissection.
static bool is_leaf(const Node& n, const Desc* d) {
  if (n.child[0] >= 0 || n.child[1] >= 0 || n.nI > 16 || n.nB > 16) return false;
  int ib[16] = {0}, bi[16] = {0};
  for (int q = 0; q < n.ndesc; ++q) {
    if (d[q].row < n.nI && d[q].col >= n.nI) ++ib[d[q].col - n.nI];
    if (d[q].row >= n.nI) {
      if (d[q].col >= n.nI) return false;
      ++bi[d[q].row - n.nI];
    }
  }
  for (int j = 0; j < n.nB; ++j)
    if (ib[j] != 1 || bi[j] != 1) return false;
  return true;
}

// Builds the tree, offsets, descriptors, maps and work lists of an nx x ny
// grid; uploads them when `to_device` (otherwise no CUDA call is made).
static int analyse(Shape& h, int nx, int ny, bool to_device) {
  h.nx = nx;
  h.ny = ny;
  std::vector<HNode> t;
  t.reserve(2 * (size_t)nx * ny / (LEAF * LEAF) + 16);
  build_tree(t, nx, ny, 0, nx, 0, ny, 0);
  const int nn = (int)t.size();
  int maxd = 0;
  for (auto& x : t) maxd = std::max(maxd, x.depth);
  h.ndepth = maxd + 1;
  h.levels.assign(h.ndepth, Level());
  std::vector<std::vector<int>> by_depth(h.ndepth);
  for (int k = 0; k < nn; ++k) by_depth[t[k].depth].push_back(k);
  std::vector<Node> dn(nn);
  long long fo = 0, vo = 0;
  double cm = 0;
  for (int d = 0; d < h.ndepth; ++d) {
    Level& L = h.levels[d];
    L.fac_lo = fo;
    long long so = 0;
    for (int k : by_depth[d]) {
      const HNode& x = t[k];
      Node& n = dn[k];
      n.nI = (int)x.I.size();
      n.nB = (int)x.B.size();
      const long long f = n.nI + n.nB;
      n.small = f <= SMALL_F ? 1 : 0;
      n.top = fo;
      n.bl = fo + (long long)n.nI * f;
      fo += (long long)n.nI * f + (long long)n.nB * n.nI;
      n.par = d & 1;
      n.s = so;
      so += (long long)n.nB * n.nB;
      n.fv = vo;
      vo += f;
      cm += (double)n.nI * f * f;
    }
    L.fac_len = fo - L.fac_lo;
    L.s_len = so;
    h.sa_pp[d & 1] = std::max(h.sa_pp[d & 1], so);
  }
  h.fac_pp = fo;
  h.fv_pp = vo;
  h.cmacs_pp = cm;
  // cells, descriptors and child maps
  std::vector<int> cells, cmap;
  std::vector<Desc> desc;
  std::vector<int> pos((size_t)nx * ny, -1);
  const int di[5] = {0, -1, 1, 0, 0}, dj[5] = {0, 0, 0, -1, 1};
  long long cnt = 0, sum = 0;
  for (int k = 0; k < nn; ++k) {
    const HNode& x = t[k];
    Node& n = dn[k];
    cnt += n.nI;
    for (int c : x.I) sum += c;
    n.cells = (int)cells.size();
    cells.insert(cells.end(), x.I.begin(), x.I.end());
    cells.insert(cells.end(), x.B.begin(), x.B.end());
    for (int q = 0; q < n.nI; ++q) pos[x.I[q]] = q;
    for (int q = 0; q < n.nB; ++q) pos[x.B[q]] = n.nI + q;
    n.desc = (int)desc.size();
    for (int q = 0; q < n.nI; ++q) {
      const int cell = x.I[q], i = cell / ny, j = cell % ny;
      for (int dir = 0; dir < 5; ++dir) {
        const int ii = i + di[dir], jj = j + dj[dir];
        if (ii < 0 || ii >= nx || jj < 0 || jj >= ny) continue;  // no periodic wrap
        const int p = pos[ii * ny + jj];
        if (p >= 0) desc.push_back(Desc{q, p, cell, dir});
      }
    }
    for (int q = 0; q < n.nB; ++q) {
      const int cell = x.B[q], i = cell / ny, j = cell % ny;
      for (int dir = 1; dir < 5; ++dir) {
        const int ii = i + di[dir], jj = j + dj[dir];
        if (ii < 0 || ii >= nx || jj < 0 || jj >= ny) continue;
        const int p = pos[ii * ny + jj];
        if (p >= 0 && p < n.nI) desc.push_back(Desc{n.nI + q, p, cell, dir});
      }
    }
    n.ndesc = (int)desc.size() - n.desc;
    for (int s = 0; s < 2; ++s) {
      n.child[s] = x.child[s];
      n.cmap[s] = -1;
      if (x.child[s] < 0) continue;
      n.cmap[s] = (int)cmap.size();
      for (int cell : t[x.child[s]].B) {
        const int p = pos[cell];
        if (p < 0) {
          set_error("nested dissection: a child's boundary cell is outside its parent's front");
          return CEV_ERR_INVALID;
        }
        cmap.push_back(p);
      }
    }
    for (int c : x.I) pos[c] = -1;
    for (int c : x.B) pos[c] = -1;
  }
  const long long nc = (long long)nx * ny;
  h.cover[0] = cnt - nc;
  h.cover[1] = sum - nc * (nc - 1) / 2;
  h.n_nodes = dn.size();
  h.n_desc = desc.size();
  // work lists per depth
  for (int d = 0; d < h.ndepth; ++d) {
    Level& L = h.levels[d];
    long long po = 0;
    for (int k : by_depth[d]) {
      Node& n = dn[k];
      const int f = n.nI + n.nB;
      n.lidx = -1;
      n.po = 0;
      if (n.small) {
        L.small.push_back(k);
        if (is_leaf(n, desc.data() + n.desc)) {
          L.leaf.push_back(k);
        } else {
          L.front.push_back(k);
          L.max_f_small = std::max(L.max_f_small, f);
          L.max_nI_small = std::max(L.max_nI_small, n.nI);
        }
        continue;
      }
      dn[k].lidx = (int)L.large.size();
      dn[k].po = (int)po;
      po += f;
      L.large.push_back(k);
      L.max_f_large = std::max(L.max_f_large, f);
      L.max_nI_large = std::max(L.max_nI_large, n.nI);
      const int nch = (f + TILE - 1) / TILE;
      for (int s = 0; s < 2; ++s)
        if (n.child[s] >= 0)
          for (int r = 0; r < dn[n.child[s]].nB; ++r) L.ext[s].push_back(make_int2(k, r));
      for (int c = 0; c < nch; ++c) L.panel.push_back(make_int2(k, c));
      const int ntiles = ((f + UT_R - 1) / UT_R) * ((f + UT_C - 1) / UT_C);
      for (int c = 0; c < ntiles; ++c) L.tiles.push_back(make_int2(k, c));
      for (int c = 0; c < (n.nB + GEMV_ROWS - 1) / GEMV_ROWS; ++c) L.gemv.push_back(make_int2(k, c));
      for (int c = 0; c < (n.nI + GEMV_ROWS - 1) / GEMV_ROWS; ++c) L.bwd.push_back(make_int2(k, c));
    }
    h.ps_pp = std::max(h.ps_pp, po * NB);
    if (!to_device) continue;
    int rc;
    if ((rc = upload(&L.d_small, L.small)) || (rc = upload(&L.d_large, L.large)) ||
        (rc = upload(&L.d_leaf, L.leaf)) || (rc = upload(&L.d_front, L.front)) ||
        (rc = upload(&L.d_ext[0], L.ext[0])) || (rc = upload(&L.d_ext[1], L.ext[1])) ||
        (rc = upload(&L.d_panel, L.panel)) || (rc = upload(&L.d_tiles, L.tiles)) ||
        (rc = upload(&L.d_gemv, L.gemv)) || (rc = upload(&L.d_bwd, L.bwd)))
      return rc;
  }
  if (!to_device) return CEV_OK;
  CEV_CUDA(cudaGetDevice(&h.device));
  int rc;
  if ((rc = upload(&h.d_nodes, dn)) || (rc = upload(&h.d_cells, cells)) ||
      (rc = upload(&h.d_cmap, cmap)) || (rc = upload(&h.d_desc, desc)))
    return rc;
  return CEV_OK;
}

// Shapes of the current device, the most recent few kept (a handle keeps its own).
static int get_shape(int nx, int ny, std::shared_ptr<Shape>& out) {
  static std::mutex mu;
  static std::vector<std::shared_ptr<Shape>> cache;
  int dev = 0;
  CEV_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  for (size_t k = 0; k < cache.size(); ++k)
    if (cache[k]->nx == nx && cache[k]->ny == ny && cache[k]->device == dev) {
      out = cache[k];
      std::rotate(cache.begin(), cache.begin() + k, cache.begin() + k + 1);  // most recent first
      return CEV_OK;
    }
  auto s = std::make_shared<Shape>();
  const int rc = analyse(*s, nx, ny, true);
  if (rc != CEV_OK) return rc;
  cache.insert(cache.begin(), s);
  if (cache.size() > 4) cache.pop_back();
  out = s;
  return CEV_OK;
}

}  // namespace nd
}  // namespace cev

using namespace cev;
using namespace cev::nd;

struct cev_nd_precond_s {
  int nx = 0, ny = 0, batch = 0, pol = 0, transpose = 0, device = 0;
  double shift = 0;
  size_t n = 0;
  std::shared_ptr<Shape> shape;
  float2* fac = nullptr;
  float2* sar[2] = {nullptr, nullptr};
  float2* fv = nullptr;
  float2* lub = nullptr;  // pivot-block LU scratch (factorisation only)
  int* lpv = nullptr;     // pivot-block permutations (factorisation only)
  float2* rb = nullptr;   // panel scratch (factorisation only)
  float2* cb = nullptr;
  int* fault = nullptr;
  const cev_fdfd_plan_s* plan = nullptr;
  ~cev_nd_precond_s() {
    cudaFree(fac); cudaFree(sar[0]); cudaFree(sar[1]); cudaFree(fv); cudaFree(lub);
    cudaFree(lpv); cudaFree(rb); cudaFree(cb);
    cudaFree(fault);
  }
};

namespace cev {
namespace nd {

static Args make_args(const cev_nd_precond_s* h, const Op& op) {
  const Shape& S = *h->shape;
  Args a;
  a.op = op;
  a.nodes = S.d_nodes;
  a.cells = S.d_cells;
  a.cmap = S.d_cmap;
  a.desc = S.d_desc;
  a.fac = h->fac;
  a.sar[0] = h->sar[0];
  a.sar[1] = h->sar[1];
  a.fv = h->fv;
  a.fault = h->fault;
  a.lub = h->lub;
  a.lpv = h->lpv;
  a.rb = h->rb;
  a.cb = h->cb;
  a.ps_pp = S.ps_pp;
  a.n = h->n;
  a.fac_pp = S.fac_pp;
  a.sa_pp[0] = S.sa_pp[0];
  a.sa_pp[1] = S.sa_pp[1];
  a.fv_pp = S.fv_pp;
  return a;
}

template <int NT, int BS>
static int launch_front(const Args& a, const Level& L, int ld, int B, cudaStream_t s) {
  const int bytes = (ld * ld + 2 * BS * ld) * (int)sizeof(float2);
  int rc = allow_dynamic_smem((const void*)k_front<NT, BS>, bytes);
  if (rc != CEV_OK) return rc;
  k_front<NT, BS><<<dim3((unsigned)L.front.size(), B), NT, bytes, s>>>(a, L.d_front, ld);
  CEV_CHECK_LAUNCH("nd k_front");
  return CEV_OK;
}

template <int NT>
static int launch_front_bs(const Args& a, const Level& L, int ld, int B, cudaStream_t s) {
  if (L.max_nI_small <= 4) return launch_front<NT, 4>(a, L, ld, B, s);
  if (L.max_nI_small <= 8) return launch_front<NT, 8>(a, L, ld, B, s);
  return launch_front<NT, 16>(a, L, ld, B, s);
}

static unsigned zero_grid(long long elems) {
  return (unsigned)std::max<long long>(1, std::min<long long>((elems + 255) / 256, 16LL * sm_count()));
}

static int factor(cev_nd_precond_s* h, const Op& op, cudaStream_t s) {
  const Args a = make_args(h, op);
  const Shape& S = *h->shape;
  const int B = h->batch;
  CEV_CUDA(cudaMemsetAsync(h->fault, 0, sizeof(int), s));
  for (int d = S.ndepth - 1; d >= 0; --d) {
    const Level& L = S.levels[d];
    if (!L.large.empty()) {
      k_zero<<<zero_grid(L.fac_len * B), 256, 0, s>>>(h->fac, S.fac_pp, L.fac_lo, L.fac_len, B);
      if (L.s_len > 0)
        k_zero<<<zero_grid(L.s_len * B), 256, 0, s>>>(h->sar[d & 1], S.sa_pp[d & 1], 0, L.s_len, B);
      CEV_CHECK_LAUNCH("nd zero");
    }
    if (!L.leaf.empty()) {
      const unsigned nl = (unsigned)L.leaf.size();
      k_leaf<<<dim3((nl + LEAF_WARPS - 1) / LEAF_WARPS, B), LEAF_WARPS * 32, 0, s>>>(a, L.d_leaf,
                                                                                   (int)nl);
      CEV_CHECK_LAUNCH("nd k_leaf");
    }
    if (!L.front.empty()) {
      // row stride: a multiple of 4 (16-byte rows of 4 x 4 tiles); NT / 2 >= ld
      const int ld = (L.max_f_small + 3) & ~3;
      int rc;
      if (ld <= 32) rc = launch_front_bs<64>(a, L, ld, B, s);
      else if (ld <= 64) rc = launch_front_bs<128>(a, L, ld, B, s);
      // fronts near 128: 8-pivot blocks keep the front plus its two panels
      // under half of an SM's shared memory, so two CTAs share an SM
      else if (ld > 96 && L.max_nI_small > 8) rc = launch_front<256, 8>(a, L, ld, B, s);
      else rc = launch_front_bs<256>(a, L, ld, B, s);
      if (rc != CEV_OK) return rc;
    }
    if (L.large.empty()) continue;
    const unsigned nl = (unsigned)L.large.size();
    {
      const int rc = allow_dynamic_smem((const void*)k_update, UPD_SMEM);
      if (rc != CEV_OK) return rc;
    }
    k_orig<<<dim3(nl, B), 256, 0, s>>>(a, L.d_large);
    for (int sl = 0; sl < 2; ++sl)
      if (!L.ext[sl].empty())
        k_extend<<<dim3((unsigned)L.ext[sl].size(), B), 128, 0, s>>>(a, L.d_ext[sl], sl);
    CEV_CHECK_LAUNCH("nd assemble");
    for (int k0 = 0; k0 < L.max_nI_large; k0 += NB) {
      k_pivblock<<<dim3((nl + 3) / 4, B), 128, 0, s>>>(a, L.d_large, (int)nl, k0);
      k_rowpanel<<<dim3((unsigned)L.panel.size(), B), TILE, 0, s>>>(a, L.d_panel, k0, (int)nl);
      k_colpanel<<<dim3((unsigned)L.panel.size(), B), TILE, 0, s>>>(a, L.d_panel, k0, (int)nl);
      k_update<<<dim3((unsigned)L.tiles.size(), B), UT_NT, UPD_SMEM, s>>>(a, L.d_tiles, k0);
    }
    CEV_CHECK_LAUNCH("nd sweep");
  }
  return CEV_OK;
}

}  // namespace nd

int nd_apply(cev_nd_precond_s* h, const float2* v, float2* z, const double* sc, int sc_stride,
             int sc_index, const KState* st, cudaStream_t s) {
  Op op{};  // entries are not needed by the apply kernels
  const nd::Args a = nd::make_args(h, op);
  const nd::Shape& S = *h->shape;
  nd::ApplyIO io{v, z, sc, sc_stride, sc_index, st};
  const int B = h->batch;
  int rc;
  for (int d = S.ndepth - 1; d >= 0; --d) {
    const nd::Level& L = S.levels[d];
    if (!L.small.empty()) {
      const unsigned ns = (unsigned)L.small.size();
      nd::k_fwd_small<<<dim3((ns + nd::WPB - 1) / nd::WPB, B), nd::WPB * 32, 0, s>>>(
          a, io, L.d_small, (int)ns);
    }
    if (!L.large.empty()) {
      const int bytes = L.max_f_large * (int)sizeof(float2);
      if ((rc = allow_dynamic_smem((const void*)nd::k_fwd_large, bytes)) != CEV_OK) return rc;
      nd::k_fwd_large<<<dim3((unsigned)L.large.size(), B), 256, bytes, s>>>(a, io, L.d_large);
      if (!L.gemv.empty()) {
        const int gb = L.max_nI_large * (int)sizeof(float2);
        if ((rc = allow_dynamic_smem((const void*)nd::k_fwd_gemv, gb)) != CEV_OK) return rc;
        nd::k_fwd_gemv<<<dim3((unsigned)L.gemv.size(), B), 256, gb, s>>>(a, io, L.d_gemv);
      }
    }
    CEV_CHECK_LAUNCH("nd forward");
  }
  for (int d = 0; d < S.ndepth; ++d) {
    const nd::Level& L = S.levels[d];
    if (!L.bwd.empty()) {
      const int bytes = L.max_f_large * (int)sizeof(float2);
      if ((rc = allow_dynamic_smem((const void*)nd::k_bwd_large, bytes)) != CEV_OK) return rc;
      nd::k_bwd_large<<<dim3((unsigned)L.bwd.size(), B), 256, bytes, s>>>(a, io, L.d_bwd);
    }
    if (!L.small.empty()) {
      const unsigned ns = (unsigned)L.small.size();
      nd::k_bwd_small<<<dim3((ns + nd::WPB - 1) / nd::WPB, B), nd::WPB * 32, 0, s>>>(
          a, io, L.d_small, (int)ns);
    }
    CEV_CHECK_LAUNCH("nd backward");
  }
  return CEV_OK;
}

int nd_check(const cev_nd_precond_s* h, const cev_fdfd_plan_s* p, int kind, int transpose) {
  CEV_REQUIRE(h != nullptr, "the direct preconditioner needs opts.direct");
  CEV_REQUIRE(h->plan == p, "direct preconditioner built for another plan");
  CEV_REQUIRE(h->transpose == transpose,
              "direct preconditioner built for transpose=%d, solve has transpose=%d", h->transpose,
              transpose);
  if (kind == CEV_PRECOND_DIRECT)
    CEV_REQUIRE(h->shift == 0.0, "CEV_PRECOND_DIRECT needs a factorisation with shift 0 (got %g)",
                h->shift);
  else
    CEV_REQUIRE(h->shift != 0.0,
                "CEV_PRECOND_SHIFTED_LAPLACIAN needs a factorisation with a non-zero shift");
  return CEV_OK;
}

}  // namespace cev

extern "C" {

int cev_nd_precond_create(cev_nd_precond* out, cev_fdfd_plan plan, const double* eps,
                          int eps_shared, int transpose, double shift, cudaStream_t stream) {
  CEV_REQUIRE(out != nullptr && plan != nullptr && eps != nullptr, "NULL argument");
  *out = nullptr;
  CEV_REQUIRE(plan->mf_nsb < 0, "multi-frequency plans have no direct preconditioner");
  CEV_REQUIRE(plan->nx >= 2 && plan->ny >= 2, "direct preconditioner needs nx, ny >= 2");
  CEV_REQUIRE((size_t)plan->nx * plan->ny < ((size_t)1 << 31), "grid too large");
  CEV_REQUIRE(std::isfinite(shift) && shift >= 0.0, "shift must be finite and >= 0");
  auto* h = new cev_nd_precond_s();
  h->nx = plan->nx;
  h->ny = plan->ny;
  h->batch = plan->batch;
  h->pol = plan->pol;
  h->transpose = transpose ? 1 : 0;
  h->shift = shift;
  h->n = plan->n();
  h->plan = plan;
  cudaGetDevice(&h->device);
  auto fail = [&](int code) {
    delete h;
    return code;
  };
  int rc = nd::get_shape(plan->nx, plan->ny, h->shape);
  if (rc != CEV_OK) return fail(rc);
  const Shape& S = *h->shape;
  const size_t B = (size_t)h->batch;
  auto alloc = [&](float2** p, size_t elems) -> int {
    if (elems == 0) return CEV_OK;
    const cudaError_t e = cudaMalloc((void**)p, sizeof(float2) * elems);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("direct preconditioner: cannot allocate %zu bytes on the device",
                sizeof(float2) * elems);
      return CEV_ERR_CUDA;
    }
    return CEV_OK;
  };
  if ((rc = alloc(&h->fac, (size_t)S.fac_pp * B)) || (rc = alloc(&h->sar[0], (size_t)S.sa_pp[0] * B)) ||
      (rc = alloc(&h->sar[1], (size_t)S.sa_pp[1] * B)) || (rc = alloc(&h->fv, (size_t)S.fv_pp * B)))
    return fail(rc);
  size_t max_large = 0;
  for (const auto& L : S.levels) max_large = std::max(max_large, L.large.size());
  if ((rc = alloc(&h->lub, max_large * B * NB * NB)) || (rc = alloc(&h->rb, (size_t)S.ps_pp * B)) ||
      (rc = alloc(&h->cb, (size_t)S.ps_pp * B)))
    return fail(rc);
  if (max_large > 0 && cudaMalloc((void**)&h->lpv, sizeof(int) * max_large * B * NB) != cudaSuccess) {
    cudaGetLastError();
    set_error("direct preconditioner: cannot allocate its pivot scratch");
    return fail(CEV_ERR_CUDA);
  }
  if (cudaMalloc((void**)&h->fault, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    set_error("direct preconditioner: cannot allocate its fault flag");
    return fail(CEV_ERR_CUDA);
  }
  const int tr = h->transpose;
  nd::Op op{plan->pol, plan->nx, plan->ny, plan->eps_complex,
            eps_shared ? (size_t)0 : plan->n(), eps, plan->cx32[tr], plan->cy32[tr],
            plan->k2_32, (float)shift};
  if ((rc = nd::factor(h, op, stream)) != CEV_OK) return fail(rc);
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return fail(cuda_status(e, "direct preconditioner factorisation"));
  int fault = 0;
  e = cudaMemcpy(&fault, h->fault, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(cuda_status(e, "direct preconditioner fault flag"));
  if (fault) {
    set_error("direct preconditioner: a zero or non-finite pivot in the complex64 factorisation");
    return fail(CEV_ERR_NUMERIC);
  }
  // the Schur arenas are only needed during the factorisation
  cudaFree(h->sar[0]);
  cudaFree(h->sar[1]);
  h->sar[0] = h->sar[1] = nullptr;
  cudaFree(h->lub);
  cudaFree(h->lpv);
  cudaFree(h->rb);
  cudaFree(h->cb);
  h->lub = nullptr;
  h->lpv = nullptr;
  h->rb = h->cb = nullptr;
  *out = h;
  return CEV_OK;
}

int cev_nd_precond_apply(cev_nd_precond h, const void* v, void* z, cudaStream_t stream) {
  CEV_REQUIRE(h != nullptr && v != nullptr && z != nullptr, "NULL argument");
  return nd_apply(h, (const float2*)v, (float2*)z, nullptr, 0, 0, nullptr, stream);
}

int cev_nd_precond_info(cev_nd_precond h, size_t* factor_bytes, double* factor_cmacs,
                        int* depths) {
  CEV_REQUIRE(h != nullptr, "NULL handle");
  if (factor_bytes) *factor_bytes = sizeof(float2) * (size_t)h->shape->fac_pp * h->batch;
  if (factor_cmacs) *factor_cmacs = h->shape->cmacs_pp * h->batch;
  if (depths) *depths = h->shape->ndepth;
  return CEV_OK;
}

int cev_nd_analyse(int nx, int ny, size_t* n_nodes, int* depths, size_t* factor_elems,
                   double* factor_cmacs, size_t* n_desc, long long* cover) {
  CEV_REQUIRE(nx >= 2 && ny >= 2 && (size_t)nx * ny < ((size_t)1 << 31), "bad grid %d x %d", nx,
              ny);
  nd::Shape h;
  const int rc = nd::analyse(h, nx, ny, false);
  if (rc != CEV_OK) return rc;
  if (n_nodes) *n_nodes = h.n_nodes;
  if (depths) *depths = h.ndepth;
  if (factor_elems) *factor_elems = (size_t)h.fac_pp;
  if (factor_cmacs) *factor_cmacs = h.cmacs_pp;
  if (n_desc) *n_desc = h.n_desc;
  if (cover) {
    cover[0] = h.cover[0];
    cover[1] = h.cover[1];
  }
  return CEV_OK;
}

int cev_nd_precond_destroy(cev_nd_precond h) {
  delete h;
  return CEV_OK;
}

}  // extern "C"
