// Incircle packing of a simplex mesh on the GPU (C ABI pg_pack_incenters of include/perigrain.h):
// the reference's get_incenter_mesh_loc (exp_dict.py:1072-1313) from the mesh its mesher returns.
//
//   element pass  incenter and inradius of every triangle (exp_dict.py:1087-1125: side lengths,
//                 length-weighted vertex mean, Heron's area, r = 2A / perimeter) or tetrahedron
//                 (:1127-1172: |det| / 6 volume, face-area weighted vertex mean, r = 6V / sum of
//                 doubled face areas), the same IEEE operations in the same order (this file is
//                 compiled with --fmad=false), so the element circles are bit-identical to numpy's.
//   adjacency     the elements of every node (get_nbd_vertex_elem, exp_dict.py:71-86) by a counting
//                 sort: per-node counts, exclusive scan, fill.
//   nodal pass    one circle per mesh node, appended after the element circles in node order:
//       plain     (:1280-1296, modify_nodal_circles = False) interior nodes only; centre = node,
//                 radius = min over its elements of |incenter - node| - inradius.
//       maximin   (:1186-1278, modify_nodal_circles = True, 2D) the problem the reference hands to
//                 GEKKO per interior node (and per boundary node with gen_bdry): maximise Z subject to
//                 Z <= |x - c_k| - r_k for the node's element circles, Z <= distance from x to the
//                 line of each boundary edge holding the node (boundary nodes), x in the bounding box
//                 of the circle centres (plus the node, for boundary nodes), started from the node
//                 (interior) or the mean of the centres and the node (boundary). Solved per node by an
//                 ascent from that initial guess to its local maximum (steepest ascent of the
//                 minimum over the eps-active constraints) followed by an exact solve of the three
//                 constraints tight there (two linear equations and one quadratic).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/perigrain.h"
#include "pg_bonds.h"
#include "pg_ieee64.cuh"

namespace pg {

namespace {

constexpr int PT = 128;       // threads per block
constexpr int PK_MAX = 16;    // element circles around one node in the maximin pass
constexpr int PL_MAX = 4;     // boundary-edge lines through one node
constexpr int PS_MAX = 12;    // constraints tight at the ascent's end considered by the exact solve

// error codes raised by the kernels (first one wins)
constexpr int32_t PE_INDEX = 1;     // element vertex or boundary index out of range
constexpr int32_t PE_ISOLATED = 2;  // a node that needs a circle belongs to no element
constexpr int32_t PE_CIRCLES = 3;   // more than PK_MAX elements around a node (maximin)
constexpr int32_t PE_LINES = 4;     // more than PL_MAX boundary edges through a node

__device__ __forceinline__ void set_err(int32_t* err, int32_t code) { atomicCAS(err, 0, code); }

// ---------------------------------------------------------------------------------------------
// element circles
// ---------------------------------------------------------------------------------------------
__global__ void k_pack_tri(const double* pos, const uint32_t* T, uint32_t ne, uint32_t nn, double* cen, double* rad,
                           uint32_t* cnt, int32_t* err) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const uint32_t ia = T[3 * (size_t)e], ib = T[3 * (size_t)e + 1], ic = T[3 * (size_t)e + 2];
  if (ia >= nn || ib >= nn || ic >= nn) {
    set_err(err, PE_INDEX);
    return;
  }
  atomicAdd(&cnt[ia], 1u);
  atomicAdd(&cnt[ib], 1u);
  atomicAdd(&cnt[ic], 1u);
  const double ax = pos[2 * (size_t)ia], ay = pos[2 * (size_t)ia + 1];
  const double bx = pos[2 * (size_t)ib], by = pos[2 * (size_t)ib + 1];
  const double cx = pos[2 * (size_t)ic], cy = pos[2 * (size_t)ic + 1];
  const double abx = bx - ax, aby = by - ay;
  const double acx = cx - ax, acy = cy - ay;
  const double bcx = cx - bx, bcy = cy - by;
  const double la = sqrt(bcx * bcx + bcy * bcy);  // side opposite a
  const double lb = sqrt(acx * acx + acy * acy);
  const double lc = sqrt(abx * abx + aby * aby);
  const double sl = la + lb + lc;
  cen[2 * (size_t)e] = (la * ax + lb * bx + lc * cx) / sl;
  cen[2 * (size_t)e + 1] = (la * ay + lb * by + lc * cy) / sl;
  const double area = 0.25 * sqrt(sl * (la - lb + lc) * (lb - lc + la) * (lc - la + lb));
  rad[e] = 2.0 * area / sl;
}

// doubled area of the face (p, q, s): the norm of the three 2x2 minors, in the order the
// reference writes them
__device__ __forceinline__ double face2(const double* p, const double* q, const double* s) {
  const double A = (p[0] - s[0]) * (p[1] - q[1]) - (p[0] - q[0]) * (p[1] - s[1]);
  const double B = (p[0] - s[0]) * (p[2] - q[2]) - (p[0] - q[0]) * (p[2] - s[2]);
  const double C = (p[1] - s[1]) * (p[2] - q[2]) - (p[1] - q[1]) * (p[2] - s[2]);
  return sqrt(A * A + B * B + C * C);
}

__global__ void k_pack_tet(const double* pos, const uint32_t* T, uint32_t ne, uint32_t nn, double* cen, double* rad,
                           uint32_t* cnt, int32_t* err) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  uint32_t v[4];
  for (int k = 0; k < 4; ++k) {
    v[k] = T[4 * (size_t)e + k];
    if (v[k] >= nn) {
      set_err(err, PE_INDEX);
      return;
    }
  }
  for (int k = 0; k < 4; ++k) atomicAdd(&cnt[v[k]], 1u);
  double p1[3], p2[3], p3[3], p4[3];
  for (int c = 0; c < 3; ++c) {
    p1[c] = pos[3 * (size_t)v[0] + c];
    p2[c] = pos[3 * (size_t)v[1] + c];
    p3[c] = pos[3 * (size_t)v[2] + c];
    p4[c] = pos[3 * (size_t)v[3] + c];
  }
  const double x1 = p1[0], y1 = p1[1], z1 = p1[2], x2 = p2[0], y2 = p2[1], z2 = p2[2];
  const double x3 = p3[0], y3 = p3[1], z3 = p3[2], x4 = p4[0], y4 = p4[1], z4 = p4[2];
  const double det = (x4 - x1) * ((y2 - y1) * (z3 - z1) - (z2 - z1) * (y3 - y1)) +
                     (y4 - y1) * ((z2 - z1) * (x3 - x1) - (x2 - x1) * (z3 - z1)) +
                     (z4 - z1) * ((x2 - x1) * (y3 - y1) - (y2 - y1) * (x3 - x1));
  const double vol = fabs((1.0 / 6.0) * det);
  const double alpha = vol * 6.0;
  const double s123 = face2(p1, p2, p3), s124 = face2(p1, p2, p4), s134 = face2(p1, p3, p4);
  const double s234 = face2(p2, p3, p4);
  const double den = s123 + s124 + s134 + s234;
  for (int c = 0; c < 3; ++c)
    cen[3 * (size_t)e + c] = (s234 * p1[c] + s134 * p2[c] + s124 * p3[c] + s123 * p4[c]) / den;
  rad[e] = alpha / den;
}

// ---------------------------------------------------------------------------------------------
// adjacency and node classes
// ---------------------------------------------------------------------------------------------
__global__ void k_pack_fill(const uint32_t* T, uint32_t ne, uint32_t nv, uint32_t nn, const uint32_t* off,
                            uint32_t* fill, uint32_t* adj) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  // an element with a vertex out of range was not counted (and has raised PE_INDEX)
  for (uint32_t k = 0; k < nv; ++k)
    if (T[(size_t)e * nv + k] >= nn) return;
  for (uint32_t k = 0; k < nv; ++k) {
    const uint32_t v = T[(size_t)e * nv + k];
    adj[off[v] + atomicAdd(&fill[v], 1u)] = e;
  }
}

__global__ void k_pack_bdry(const uint32_t* bn, uint32_t nb, uint32_t nn, uint32_t* mask, int32_t* err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  if (bn[k] >= nn) {
    set_err(err, PE_INDEX);
    return;
  }
  mask[bn[k]] = 1;
}

__global__ void k_pack_bedges(const uint32_t* be, uint32_t nbe, uint32_t nn, uint32_t* bcnt, uint32_t* bedge,
                              int32_t* err) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nbe) return;
  for (int s = 0; s < 2; ++s) {
    const uint32_t v = be[2 * (size_t)k + s];
    if (v >= nn) {
      set_err(err, PE_INDEX);
      return;
    }
    const uint32_t j = atomicAdd(&bcnt[v], 1u);
    if (j < (uint32_t)PL_MAX) bedge[(size_t)v * PL_MAX + j] = k;
    else set_err(err, PE_LINES);
  }
}

// which nodes get a circle: interior nodes, plus boundary nodes when `all_bdry`
__global__ void k_pack_flags(uint32_t nn, const uint32_t* mask, int all_bdry, uint32_t* flag) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nn) flag[i] = (!mask[i] || all_bdry) ? 1u : 0u;
}

// ---------------------------------------------------------------------------------------------
// plain nodal circles
// ---------------------------------------------------------------------------------------------
template <int D>
__global__ void k_pack_plain(const double* pos, uint32_t nn, uint32_t ne, const double* cen, const double* rad,
                             const uint32_t* off, const uint32_t* adj, const uint32_t* flag, const uint32_t* rank,
                             double* ocen, double* orad, int32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn || !flag[i]) return;
  const uint32_t b = off[i], e = off[i + 1];
  if (b == e) {
    set_err(err, PE_ISOLATED);
    return;
  }
  double x[D];
  for (int c = 0; c < D; ++c) x[c] = pos[(size_t)i * D + c];
  double m = 0.0;
  bool nan = false;
  for (uint32_t k = b; k < e; ++k) {
    const uint32_t t = adj[k];
    double s = 0.0;
    for (int c = 0; c < D; ++c) {
      const double d = cen[(size_t)t * D + c] - x[c];
      s = (c == 0) ? d * d : s + d * d;
    }
    const double v = sqrt(s) - rad[t];
    if (v != v) nan = true;
    if (k == b || v < m) m = v;
  }
  const uint32_t o = ne + rank[i];
  for (int c = 0; c < D; ++c) ocen[(size_t)o * D + c] = x[c];
  orad[o] = nan ? (double)NAN : m;
}

// ---------------------------------------------------------------------------------------------
// maximin nodal circles (2D)
// ---------------------------------------------------------------------------------------------
// One thread per node, MM_T threads per block. A thread's problem -- its circles, lines and the
// gradients of the ascent -- lives in its own column of the block's shared memory, so the kernel
// keeps almost nothing in local memory. Coordinates are shifted to the initial guess and scaled by
// the box extent L, so the solve works on numbers of order one.
constexpr int MM_T = 32;
constexpr int R_CX = 0, R_CY = R_CX + PK_MAX, R_CR = R_CY + PK_MAX;           // circles
constexpr int R_AX = R_CR + PK_MAX, R_AY = R_AX + PL_MAX, R_AB = R_AY + PL_MAX;  // lines |ax x + ay y + ab|
constexpr int R_GX = R_AB + PL_MAX, R_GY = R_GX + PK_MAX + PL_MAX;              // ascent gradients
constexpr int MM_ROWS = R_GY + PK_MAX + PL_MAX;

struct MaxiMin {
  double (*sm)[MM_T];  // shared rows, column t
  int t, nc, nl;
  double lo[2], hi[2];  // box
  __device__ __forceinline__ double& at(int row, int k) const { return sm[row + k][t]; }
};

__device__ __forceinline__ double mm_value(const MaxiMin& M, double x, double y) {
  double m = INFINITY;
  for (int k = 0; k < M.nc; ++k) {
    const double cx = M.at(R_CX, k), cy = M.at(R_CY, k);
    m = fmin(m, ieee64::sqrt_rn((x - cx) * (x - cx) + (y - cy) * (y - cy)) - M.at(R_CR, k));
  }
  for (int l = 0; l < M.nl; ++l) m = fmin(m, fabs(M.at(R_AX, l) * x + M.at(R_AY, l) * y + M.at(R_AB, l)));
  return m;
}

__device__ __forceinline__ double clampd(double v, double lo, double hi) { return fmin(fmax(v, lo), hi); }

// minimum-norm point of the convex hull of the n gradients in rows R_GX / R_GY (0 when the hull
// holds the origin)
__device__ __forceinline__ void min_norm(const MaxiMin& M, int n, double* ox, double* oy) {
  double bx = 0.0, by = 0.0, bn = INFINITY;
  for (int i = 0; i < n; ++i) {
    const double gix = M.at(R_GX, i), giy = M.at(R_GY, i);
    const double n2 = gix * gix + giy * giy;
    if (n2 < bn) {
      bn = n2;
      bx = gix;
      by = giy;
    }
    for (int j = i + 1; j < n; ++j) {
      const double dx = M.at(R_GX, j) - gix, dy = M.at(R_GY, j) - giy;
      const double dd = dx * dx + dy * dy;
      if (dd <= 0.0) continue;
      const double t = clampd(ieee64::div_rn(-(gix * dx + giy * dy), dd), 0.0, 1.0);
      const double px = gix + t * dx, py = giy + t * dy;
      const double p2 = px * px + py * py;
      if (p2 < bn) {
        bn = p2;
        bx = px;
        by = py;
      }
    }
  }
  // p is the hull's closest point to the origin iff p . (g - p) >= 0 for every g
  for (int i = 0; i < n; ++i)
    if (bx * (M.at(R_GX, i) - bx) + by * (M.at(R_GY, i) - by) < -1e-12) {
      bx = 0.0;
      by = 0.0;
      break;
    }
  *ox = bx;
  *oy = by;
}

// Ascent from the origin (the initial guess) to a local maximum of the minimum over the
// constraints; returns the value, the point in (*px, *py) and the final step in *step_out.
__device__ __forceinline__ double mm_ascent(const MaxiMin& M, double* px, double* py, double* step_out) {
  double x = clampd(0.0, M.lo[0], M.hi[0]), y = clampd(0.0, M.lo[1], M.hi[1]);
  double fx = mm_value(M, x, y);
  double step = 0.25;
  // the ascent only has to bring the point within reach of the exact solve, which takes the
  // constraints within max(1e-6, 8 step) of the minimum; stopping at step 1e-7 (instead of running
  // to 1e-13) halves the iterations and leaves every solved circle unchanged on the test meshes
  for (int it = 0; it < 6000 && step > 1e-7; ++it) {
    // gradients of the constraints within `step` of the minimum: moving by step / 2 along the
    // min-norm direction of their hull raises all of them, and no other one can drop below fx
    int n = 0;
    for (int k = 0; k < M.nc; ++k) {
      const double dx = x - M.at(R_CX, k), dy = y - M.at(R_CY, k);
      const double d = ieee64::sqrt_rn(dx * dx + dy * dy);
      if (d - M.at(R_CR, k) <= fx + step && d > 0.0) {
        const ieee64::Divisor dd = ieee64::make_divisor(d);
        M.at(R_GX, n) = ieee64::div_rn(dx, dd);
        M.at(R_GY, n) = ieee64::div_rn(dy, dd);
        ++n;
      }
    }
    for (int l = 0; l < M.nl; ++l) {
      const double s = M.at(R_AX, l) * x + M.at(R_AY, l) * y + M.at(R_AB, l);
      if (fabs(s) <= fx + step) {
        const double sg = s < 0.0 ? -1.0 : 1.0;
        M.at(R_GX, n) = sg * M.at(R_AX, l);
        M.at(R_GY, n) = sg * M.at(R_AY, l);
        ++n;
      }
    }
    double dx = 0.0, dy = 0.0;
    if (n) min_norm(M, n, &dx, &dy);
    // box faces: no motion through a face the point sits on
    if ((x <= M.lo[0] && dx < 0.0) || (x >= M.hi[0] && dx > 0.0)) dx = 0.0;
    if ((y <= M.lo[1] && dy < 0.0) || (y >= M.hi[1] && dy > 0.0)) dy = 0.0;
    const double nd = ieee64::sqrt_rn(dx * dx + dy * dy);
    if (nd < 1e-12) {
      step *= 0.5;
      continue;
    }
    const double s = ieee64::div_rn(0.5 * step, nd);
    const double nx = clampd(x + s * dx, M.lo[0], M.hi[0]), ny = clampd(y + s * dy, M.lo[1], M.hi[1]);
    const double fn = mm_value(M, nx, ny);
    if (fn > fx) {
      x = nx;
      y = ny;
      fx = fn;
      step = fmin(step * 1.5, 0.25);
    } else {
      step *= 0.5;
    }
  }
  *px = x;
  *py = y;
  *step_out = step;
  return fx;
}

// One constraint of the exact solve, packed in 32 bits: kind << 8 | idx, plus bit 16 = negative
// side (lines) or upper face (box). kind 0 circle, 1 line, 2 box face (idx = axis).
constexpr uint32_t PC_CIRCLE = 0, PC_LINE = 1, PC_BOX = 2, PC_NEG = 1u << 16;
__device__ __forceinline__ uint32_t pc_kind(uint32_t p) { return (p >> 8) & 0xffu; }
__device__ __forceinline__ int pc_idx(uint32_t p) { return (int)(p & 0xffu); }

// linear row r . (x, y, Z) = rhs of a line or box piece
__device__ __forceinline__ void piece_row(const MaxiMin& M, uint32_t p, double* r, double* rhs) {
  if (pc_kind(p) == PC_LINE) {
    const double sg = (p & PC_NEG) ? -1.0 : 1.0;
    const int l = pc_idx(p);
    r[0] = sg * M.at(R_AX, l);
    r[1] = sg * M.at(R_AY, l);
    r[2] = -1.0;
    *rhs = -sg * M.at(R_AB, l);
  } else {
    const int a = pc_idx(p);
    r[0] = a == 0 ? 1.0 : 0.0;
    r[1] = a == 1 ? 1.0 : 0.0;
    r[2] = 0.0;
    *rhs = (p & PC_NEG) ? M.hi[a] : M.lo[a];
  }
}

__device__ __forceinline__ double det3(const double (&A)[3][3]) {
  return A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
         A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
}

// points where the three pieces are tight; returns how many (0..2) were written to (qx, qy, qz)
__device__ __forceinline__ int solve_triple(const MaxiMin& M, const uint32_t (&P)[3], double (&qx)[2],
                                            double (&qy)[2], double (&qz)[2]) {
  int circ[3] = {0, 0, 0}, nc = 0;
  double R[3][3], rhs[3];
  int nr = 0;
  for (int k = 0; k < 3; ++k)
    if (pc_kind(P[k]) == PC_CIRCLE) circ[nc++] = pc_idx(P[k]);
  for (int k = 0; k < 3; ++k)
    if (pc_kind(P[k]) != PC_CIRCLE) {
      piece_row(M, P[k], R[nr], &rhs[nr]);
      ++nr;
    }
  if (nc == 0) {
    const double det = det3(R);
    if (fabs(det) < 1e-14) return 0;
    double sol[3];
    for (int c = 0; c < 3; ++c) {
      double A[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) A[i][j] = (j == c) ? rhs[i] : R[i][j];
      sol[c] = det3(A) / det;
    }
    qx[0] = sol[0];
    qy[0] = sol[1];
    qz[0] = sol[2];
    return 1;
  }
  // differences of the circle equations against the first circle are linear in (x, y, Z)
  const int c1 = circ[0];
  const double p1x = M.at(R_CX, c1), p1y = M.at(R_CY, c1), r1 = M.at(R_CR, c1);
  for (int k = 1; k < nc; ++k) {
    const int cj = circ[k];
    const double pjx = M.at(R_CX, cj), pjy = M.at(R_CY, cj), rj = M.at(R_CR, cj);
    R[nr][0] = 2.0 * (pjx - p1x);
    R[nr][1] = 2.0 * (pjy - p1y);
    R[nr][2] = 2.0 * (rj - r1);
    rhs[nr] = (pjx * pjx + pjy * pjy - rj * rj) - (p1x * p1x + p1y * p1y - r1 * r1);
    ++nr;
  }
  // nr == 2: solutions Q0 + t * Dir, Dir = R0 x R1, Q0 the least-norm solution
  const double Dx = R[0][1] * R[1][2] - R[0][2] * R[1][1];
  const double Dy = R[0][2] * R[1][0] - R[0][0] * R[1][2];
  const double Dz = R[0][0] * R[1][1] - R[0][1] * R[1][0];
  const double g00 = R[0][0] * R[0][0] + R[0][1] * R[0][1] + R[0][2] * R[0][2];
  const double g01 = R[0][0] * R[1][0] + R[0][1] * R[1][1] + R[0][2] * R[1][2];
  const double g11 = R[1][0] * R[1][0] + R[1][1] * R[1][1] + R[1][2] * R[1][2];
  const double gd = g00 * g11 - g01 * g01;
  if (Dx * Dx + Dy * Dy + Dz * Dz < 1e-24 || fabs(gd) < 1e-24) return 0;
  const double u0 = (g11 * rhs[0] - g01 * rhs[1]) / gd, u1 = (g00 * rhs[1] - g01 * rhs[0]) / gd;
  const double q0x = u0 * R[0][0] + u1 * R[1][0], q0y = u0 * R[0][1] + u1 * R[1][1], q0z = u0 * R[0][2] + u1 * R[1][2];
  const double ex = q0x - p1x, ey = q0y - p1y, ez = q0z + r1;
  const double a = Dx * Dx + Dy * Dy - Dz * Dz, b = 2.0 * (ex * Dx + ey * Dy - ez * Dz), c = ex * ex + ey * ey - ez * ez;
  double t[2] = {0.0, 0.0};
  int nt = 0;
  if (fabs(a) < 1e-14) {
    if (fabs(b) < 1e-300) return 0;
    t[nt++] = -c / b;
  } else {
    double disc = b * b - 4.0 * a * c;
    if (disc < 0.0) {
      if (disc < -1e-12 * (b * b + fabs(4.0 * a * c))) return 0;
      disc = 0.0;
    }
    const double q = -0.5 * (b + copysign(sqrt(disc), b));
    t[nt++] = q / a;
    if (q != 0.0) t[nt++] = c / q;
  }
  int w = 0;
  for (int k = 0; k < nt; ++k) {
    const double zx = q0x + t[k] * Dx, zy = q0y + t[k] * Dy, zz = q0z + t[k] * Dz;
    bool ok = true;
    for (int j = 0; j < nc; ++j) ok = ok && (zz + M.at(R_CR, circ[j]) >= -1e-12);  // external tangency
    if (!ok) continue;
    qx[w] = zx;
    qy[w] = zy;
    qz[w] = zz;
    ++w;
  }
  return w;
}

__global__ void __launch_bounds__(MM_T) k_pack_maximin(const double* pos, uint32_t nn, uint32_t ne, const double* cen,
                                                       const double* rad, const uint32_t* off, const uint32_t* adj,
                                                       const uint32_t* flag, const uint32_t* rank, const uint32_t* mask,
                                                       const uint32_t* bcnt, const uint32_t* bedge, const uint32_t* be,
                                                       double* ocen, double* orad, int32_t* err, uint32_t* unpolished) {
  __shared__ double sm[MM_ROWS][MM_T];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn || !flag[i]) return;
  const uint32_t b = off[i], e = off[i + 1];
  if (b == e) {
    set_err(err, PE_ISOLATED);
    return;
  }
  if (e - b > (uint32_t)PK_MAX) {
    set_err(err, PE_CIRCLES);
    return;
  }
  MaxiMin M;
  M.sm = sm;
  M.t = (int)threadIdx.x;
  const bool bdry = mask[i] != 0;
  const double nx = pos[2 * (size_t)i], ny = pos[2 * (size_t)i + 1];
  // the node's elements in ascending order (the fill order is not deterministic), kept in the
  // circle rows as doubles until the coordinates replace them
  const int ncir = (int)(e - b);
  for (int k = 0; k < ncir; ++k) {
    const double t = (double)adj[b + k];
    int j = k;
    while (j > 0 && M.at(R_CR, j - 1) > t) {
      M.at(R_CR, j) = M.at(R_CR, j - 1);
      --j;
    }
    M.at(R_CR, j) = t;
  }
  // box and initial guess in the reference's terms (exp_dict.py:1196-1199 interior, :1250-1260
  // boundary)
  double lo[2] = {INFINITY, INFINITY}, hi[2] = {-INFINITY, -INFINITY}, sx = 0.0, sy = 0.0;
  for (int k = 0; k < ncir; ++k) {
    const uint32_t t = (uint32_t)M.at(R_CR, k);
    const double px = cen[2 * (size_t)t], py = cen[2 * (size_t)t + 1];
    lo[0] = fmin(lo[0], px);
    hi[0] = fmax(hi[0], px);
    lo[1] = fmin(lo[1], py);
    hi[1] = fmax(hi[1], py);
    sx += px;
    sy += py;
  }
  double x0 = nx, y0 = ny;
  if (bdry) {
    lo[0] = fmin(lo[0], nx);
    hi[0] = fmax(hi[0], nx);
    lo[1] = fmin(lo[1], ny);
    hi[1] = fmax(hi[1], ny);
    x0 = (sx + nx) / (double)(e - b + 1);
    y0 = (sy + ny) / (double)(e - b + 1);
  }
  const double L = fmax(fmax(hi[0] - lo[0], hi[1] - lo[1]), 1e-300);
  const double iL = 1.0 / L;
  M.nc = ncir;
  for (int k = 0; k < ncir; ++k) {
    const uint32_t t = (uint32_t)M.at(R_CR, k);
    M.at(R_CX, k) = (cen[2 * (size_t)t] - x0) * iL;
    M.at(R_CY, k) = (cen[2 * (size_t)t + 1] - y0) * iL;
    M.at(R_CR, k) = rad[t] * iL;
  }
  M.nl = 0;
  if (bdry) {
    // boundary edges through the node in ascending order
    const uint32_t nb = min(bcnt[i], (uint32_t)PL_MAX);
    uint32_t eds[PL_MAX] = {0, 0, 0, 0};
    for (uint32_t k = 0; k < nb; ++k) {
      const uint32_t t = bedge[(size_t)i * PL_MAX + k];
      uint32_t j = k;
      while (j > 0 && eds[j - 1] > t) {
        eds[j] = eds[j - 1];
        --j;
      }
      eds[j] = t;
    }
    for (uint32_t k = 0; k < nb; ++k) {
      const uint32_t ed = eds[k];
      const uint32_t v1 = be[2 * (size_t)ed], v2 = be[2 * (size_t)ed + 1];
      const double e1x = pos[2 * (size_t)v1], e1y = pos[2 * (size_t)v1 + 1];
      const double ux = pos[2 * (size_t)v2] - e1x, uy = pos[2 * (size_t)v2 + 1] - e1y;
      const double un = sqrt(ux * ux + uy * uy);
      if (!(un > 0.0)) continue;
      // |u x (p - e1)| / |u| (exp_dict.py:1240-1247) = |n . (p - e1)|, n = (-uy, ux) / |u|
      const double ax = -uy / un, ay = ux / un;
      M.at(R_AX, M.nl) = ax;
      M.at(R_AY, M.nl) = ay;
      M.at(R_AB, M.nl) = (ax * (x0 - e1x) + ay * (y0 - e1y)) * iL;
      ++M.nl;
    }
  }
  M.lo[0] = (lo[0] - x0) * iL;
  M.hi[0] = (hi[0] - x0) * iL;
  M.lo[1] = (lo[1] - y0) * iL;
  M.hi[1] = (hi[1] - y0) * iL;

  double x = 0.0, y = 0.0, step = 0.0;
  const double fx = mm_ascent(M, &x, &y, &step);
  // exact solve: constraints within `near` of the minimum (and box faces within `near`) at the
  // ascent's end; the tight point with value >= fx closest to the ascent's end is the maximum
  const double near = fmax(1e-6, 8.0 * step);
  uint32_t S[PS_MAX];
  int ns = 0;
  for (int k = 0; k < M.nc && ns < PS_MAX; ++k) {
    const double dx = x - M.at(R_CX, k), dy = y - M.at(R_CY, k);
    const double v = sqrt(dx * dx + dy * dy) - M.at(R_CR, k);
    if (v <= fx + near) S[ns++] = (PC_CIRCLE << 8) | (uint32_t)k;
  }
  for (int l = 0; l < M.nl && ns < PS_MAX; ++l) {
    const double s = M.at(R_AX, l) * x + M.at(R_AY, l) * y + M.at(R_AB, l);
    if (fabs(s) <= fx + near) S[ns++] = (PC_LINE << 8) | (uint32_t)l | (s < 0.0 ? PC_NEG : 0u);
  }
  for (int a = 0; a < 2 && ns < PS_MAX; ++a) {
    const double w = a == 0 ? x : y;
    if (w - M.lo[a] <= near && ns < PS_MAX) S[ns++] = (PC_BOX << 8) | (uint32_t)a;
    if (M.hi[a] - w <= near && ns < PS_MAX) S[ns++] = (PC_BOX << 8) | (uint32_t)a | PC_NEG;
  }
  double bx = x, by = y, bf = fx, bd = INFINITY;
  for (int p = 0; p < ns; ++p)
    for (int q = p + 1; q < ns; ++q)
      for (int r = q + 1; r < ns; ++r) {
        const uint32_t T3[3] = {S[p], S[q], S[r]};
        int boxes = 0, axes = 0;
        for (int k = 0; k < 3; ++k)
          if (pc_kind(T3[k]) == PC_BOX) {
            ++boxes;
            axes |= 1 << pc_idx(T3[k]);
          }
        if (boxes == 3 || (boxes == 2 && axes != 3)) continue;
        double qx[2], qy[2], qz[2];
        const int nq = solve_triple(M, T3, qx, qy, qz);
        for (int k = 0; k < nq; ++k) {
          const double tol = 1e-11;
          if (qx[k] < M.lo[0] - tol || qx[k] > M.hi[0] + tol || qy[k] < M.lo[1] - tol || qy[k] > M.hi[1] + tol) continue;
          const double cxk = clampd(qx[k], M.lo[0], M.hi[0]), cyk = clampd(qy[k], M.lo[1], M.hi[1]);
          const double v = mm_value(M, cxk, cyk);
          if (boxes < 2 && fabs(v - qz[k]) > 1e-9) continue;  // another constraint is lower there
          if (v < fx - 1e-12) continue;
          const double d = (cxk - x) * (cxk - x) + (cyk - y) * (cyk - y);
          if (d < bd) {
            bd = d;
            bx = cxk;
            by = cyk;
            bf = v;
          }
        }
      }
  if (bd == INFINITY) atomicAdd(unpolished, 1u);
  const uint32_t o = ne + rank[i];
  ocen[2 * (size_t)o] = x0 + bx * L;
  ocen[2 * (size_t)o + 1] = y0 + by * L;
  orad[o] = bf * L;
}

inline uint32_t cdivp(uint64_t a, uint32_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

}  // namespace pg

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
namespace {
thread_local std::string g_pack_err;

int pack_fail(int code, const std::string& msg) {
  g_pack_err = msg;
  return code;
}
}  // namespace

extern "C" const char* pg_pack_last_error(void) { return g_pack_err.c_str(); }

extern "C" int pg_pack_incenters(const pg_pack_mesh* m, int32_t modify_nodal_circles, int32_t gen_bdry,
                                 double* centers, double* radii, uint32_t* n_out, uint32_t* n_unpolished,
                                 void* stream) {
  using namespace pg;
  if (!m || !n_out || !centers || !radii) return pack_fail(PG_EINVAL, "null argument");
  *n_out = 0;
  if (n_unpolished) *n_unpolished = 0;
  const uint32_t D = m->dim, nn = m->n_nodes, ne = m->n_elems, nv = D + 1;
  if (D != 2 && D != 3) return pack_fail(PG_EINVAL, "dim must be 2 or 3");
  if (modify_nodal_circles && D != 2) return pack_fail(PG_EINVAL, "modified nodal circles are defined for 2D meshes");
  if ((nn && !m->pos) || (ne && !m->elems) || (m->n_bdry_nodes && !m->bdry_nodes) ||
      (m->n_bdry_edges && !m->bdry_edges))
    return pack_fail(PG_EINVAL, "null mesh array");
  if (ne == 0) return PG_OK;
  if (nn == 0) return pack_fail(PG_EINVAL, "elements without nodes");
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t tiles = bond_scan_tiles(nn);
  // scratch (u32 words): cnt, off[nn+1], fill, mask, bcnt, bedge[nn*PL_MAX], flag, rank[nn+1],
  // adj[ne*nv], tile_sum, done, err, unpolished
  const size_t words = (size_t)nn * (7 + PL_MAX) + 2 + (size_t)ne * nv + tiles + 3;
  void* block = nullptr;
  cudaError_t e = cudaMalloc(&block, words * 4);
  if (e != cudaSuccess) return pack_fail(PG_ENOMEM, cudaGetErrorString(e));
  uint32_t* w = (uint32_t*)block;
  uint32_t *cnt = w, *off = cnt + nn, *fill = off + nn + 1, *mask = fill + nn, *bcnt = mask + nn;
  uint32_t *bedge = bcnt + nn, *flag = bedge + (size_t)nn * PL_MAX, *rank = flag + nn;
  uint32_t *adj = rank + nn + 1, *tsum = adj + (size_t)ne * nv, *done = tsum + tiles;
  int32_t* err = (int32_t*)(done + 1);
  uint32_t* unpol = done + 2;
  int rc = PG_OK;
  int32_t derr = 0;
  uint32_t unp = 0;
  e = cudaMemsetAsync(block, 0, words * 4, st);
  if (e == cudaSuccess) {
    if (D == 2) {
      k_pack_tri<<<cdivp(ne, PT), PT, 0, st>>>(m->pos, m->elems, ne, nn, centers, radii, cnt, err);
    } else {
      k_pack_tet<<<cdivp(ne, PT), PT, 0, st>>>(m->pos, m->elems, ne, nn, centers, radii, cnt, err);
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = scan_u32_dev(cnt, nn, off, tsum, done, st);
  if (e == cudaSuccess) {
    k_pack_fill<<<cdivp(ne, PT), PT, 0, st>>>(m->elems, ne, nv, nn, off, fill, adj);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && m->n_bdry_nodes) {
    k_pack_bdry<<<cdivp(m->n_bdry_nodes, PT), PT, 0, st>>>(m->bdry_nodes, m->n_bdry_nodes, nn, mask, err);
    e = cudaGetLastError();
  }
  const bool maximin = modify_nodal_circles != 0;
  const bool all_bdry = maximin && gen_bdry;
  if (e == cudaSuccess && all_bdry && m->n_bdry_edges) {
    k_pack_bedges<<<cdivp(m->n_bdry_edges, PT), PT, 0, st>>>(m->bdry_edges, m->n_bdry_edges, nn, bcnt, bedge, err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    k_pack_flags<<<cdivp(nn, PT), PT, 0, st>>>(nn, mask, all_bdry ? 1 : 0, flag);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = scan_u32_dev(flag, nn, rank, tsum, done, st);
  // the element pass must be error-free before the nodal pass reads the adjacency
  if (e == cudaSuccess) e = cudaMemcpyAsync(&derr, err, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess && derr == 0) {
    if (maximin) {
      k_pack_maximin<<<cdivp(nn, MM_T), MM_T, 0, st>>>(m->pos, nn, ne, centers, radii, off, adj, flag, rank, mask, bcnt,
                                                   bedge, m->bdry_edges, centers, radii, err, unpol);
    } else if (D == 2) {
      k_pack_plain<2><<<cdivp(nn, PT), PT, 0, st>>>(m->pos, nn, ne, centers, radii, off, adj, flag, rank, centers,
                                                     radii, err);
    } else {
      k_pack_plain<3><<<cdivp(nn, PT), PT, 0, st>>>(m->pos, nn, ne, centers, radii, off, adj, flag, rank, centers,
                                                     radii, err);
    }
    e = cudaGetLastError();
  }
  uint32_t total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, rank + nn, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&derr, err, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&unp, unpol, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    rc = pack_fail(PG_ECUDA, cudaGetErrorString(e));
  } else if (derr == PE_INDEX) {
    rc = pack_fail(PG_EINVAL, "node index out of range in elems, bdry_nodes or bdry_edges");
  } else if (derr == PE_ISOLATED) {
    rc = pack_fail(PG_EINVAL, "a node that needs a circle belongs to no element");
  } else if (derr == PE_CIRCLES) {
    rc = pack_fail(PG_ECAPACITY, "more than 16 elements around one node");
  } else if (derr == PE_LINES) {
    rc = pack_fail(PG_ECAPACITY, "more than 4 boundary edges through one node");
  } else {
    *n_out = ne + total;
    if (n_unpolished) *n_unpolished = unp;
  }
  cudaFree(block);
  return rc;
}
