// Host-side mesh substrate: Ac mesh, combined AaAc mesh, neighbour functions and the
// five-colouring, built from a base triangulation.
//
// Follows, step for step where the result depends on it:
//   make_Ac_mesh                      mesh_ArakawaC_module.f90:24-241
//   find_Ac_edge_indices              mesh_ArakawaC_module.f90:242-285
//   make_combined_AaAc_mesh           mesh_ArakawaC_module.f90:286-540
//   get_neighbour_functions(_vertex_gr) mesh_derivatives_module.f90:14-313
//   calculate_five_colouring_AaAc     mesh_five_colour_module.f90:18-735
// The Ac numbering, the AaAc connectivity and the colouring are integer results that
// must be identical to the reference's; the neighbour-function arithmetic keeps the
// reference's expression order (this file is built with -ffp-contract=off).
//
// The colouring keeps the reference's queue discipline (append on add, order-preserving
// removal, top = last entry, "return v to the rear of Q5" = move last to first) but
// stores Q4 and Q5 as doubly linked lists, so every queue operation is O(1) instead of
// the O(n) array shifts of the Fortran code.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/ufemism_gb300.h"
#include "ufe_internal.h"

namespace ufe {
namespace {

struct Col {  // column-major view of a Fortran array, 0-based row/col arguments
  template <class T>
  static T &at(T *p, int64_t ld, int64_t i, int64_t j) { return p[i + j * ld]; }
};

bool boundary_segment(const int32_t *edge, int v1, int v2) {
  const int e1 = edge[v1], e2 = edge[v2];
  if (e1 == 0 || e2 == 0) return false;
  // Edge codes adjacent along the boundary walk N(1) NE(2) E(3) SE(4) S(5) SW(6) W(7) NW(8):
  // odd codes (sides) accept their two corners and themselves; corners accept the two
  // sides they join and the corners at the far end of those sides.
  static const uint16_t accept[9] = {
      0,
      (1u << 8) | (1u << 1) | (1u << 2),
      (1u << 8) | (1u << 1) | (1u << 2) | (1u << 3) | (1u << 4),
      (1u << 2) | (1u << 3) | (1u << 4),
      (1u << 2) | (1u << 3) | (1u << 4) | (1u << 5) | (1u << 6),
      (1u << 4) | (1u << 5) | (1u << 6),
      (1u << 4) | (1u << 5) | (1u << 6) | (1u << 7) | (1u << 8),
      (1u << 6) | (1u << 7) | (1u << 8),
      (1u << 6) | (1u << 7) | (1u << 8) | (1u << 1) | (1u << 2),
  };
  if (e1 < 1 || e1 > 8 || e2 < 1 || e2 > 8) return false;
  return (accept[e1] >> e2) & 1u;
}

}  // namespace

// Averaged-gradient neighbour functions of one vertex (Berends et al. 2021, Eqs. A1-A25),
// in the order of get_neighbour_functions_vertex_gr. px/py: home coordinates; qx/qy: the
// n neighbours in CCW order. Outputs have n+1 entries, home last.
void neighbour_functions(double px, double py, int n, const double *qx, const double *qy,
                         bool edge, double *Nx, double *Ny, double *Nxx, double *Nxy,
                         double *Nyy) {
  double tx[kMaxDeg][3], ty[kMaxDeg][3], sx[kMaxDeg][3], sy[kMaxDeg][3];
  for (int k = 0; k <= n; ++k) Nx[k] = Ny[k] = Nxx[k] = Nxy[k] = Nyy[k] = 0.0;
  const int ntri = edge ? n - 1 : n;
  const int nsub = edge ? n - 2 : n;
  auto wrap = [n](int k) { return k >= n ? k - n : k; };
  for (int t = 0; t < ntri; ++t) {  // first-order functions on the fan triangles (A1, A3)
    const int t1 = wrap(t + 1);
    const double xt = qx[t], yt = qy[t], xu = qx[t1], yu = qy[t1];
    const double nz = ((xt - px) * (yu - py)) - ((yt - py) * (xu - px));
    tx[t][0] = (yt - yu) / nz;
    tx[t][1] = (yu - py) / nz;
    tx[t][2] = (py - yt) / nz;
    ty[t][0] = (xu - xt) / nz;
    ty[t][1] = (px - xu) / nz;
    ty[t][2] = (xt - px) / nz;
  }
  for (int s = 0; s < nsub; ++s) {  // sub-triangles through the fan-triangle centroids (A11, A13)
    const int s1 = wrap(s + 1), s2 = wrap(s1 + 1);
    const double xs = qx[s], ys = qy[s], x1 = qx[s1], y1 = qy[s1], x2 = qx[s2], y2 = qy[s2];
    const double nz = (((1.0 / 3.0) * ((xs + x1) - 2.0 * px)) * ((y1 + y2) - 2.0 * py)) -
                      (((1.0 / 3.0) * ((ys + y1) - 2.0 * py)) * ((x1 + x2) - 2.0 * px));
    sx[s][0] = (ys - y2) / nz;
    sx[s][1] = ((y1 + y2) - 2.0 * py) / nz;
    sx[s][2] = ((2.0 * py - ys) - y1) / nz;
    sy[s][0] = (x2 - xs) / nz;
    sy[s][1] = ((2.0 * px - x1) - x2) / nz;
    sy[s][2] = ((xs + x1) - 2.0 * px) / nz;
  }
  if (!edge) {
    const double w = 1.0 / (double)n;
    double a = 0.0, b = 0.0;
    for (int t = 0; t < n; ++t) a = a + tx[t][0];
    for (int t = 0; t < n; ++t) b = b + ty[t][0];
    Nx[n] = w * a;  // A7a
    Ny[n] = w * b;
    for (int c = 0; c < n; ++c) {  // A7b
      const int cm = c == 0 ? n - 1 : c - 1;
      Nx[c] = w * (tx[c][1] + tx[cm][2]);
      Ny[c] = w * (ty[c][1] + ty[cm][2]);
    }
    for (int s = 0; s < n; ++s) {  // A23a-c
      const int s1 = wrap(s + 1);
      Nxx[n] = Nxx[n] + (w * (((sx[s][0] * Nx[n]) + (sx[s][1] * tx[s][0])) + (sx[s][2] * tx[s1][0])));
      Nxy[n] = Nxy[n] + (w * (((sy[s][0] * Nx[n]) + (sy[s][1] * tx[s][0])) + (sy[s][2] * tx[s1][0])));
      Nyy[n] = Nyy[n] + (w * (((sy[s][0] * Ny[n]) + (sy[s][1] * ty[s][0])) + (sy[s][2] * ty[s1][0])));
    }
    double sx1 = 0.0, sy1 = 0.0;
    for (int s = 0; s < n; ++s) sx1 = sx1 + sx[s][0];
    for (int s = 0; s < n; ++s) sy1 = sy1 + sy[s][0];
    for (int s = 0; s < n; ++s) {  // A23d-f
      const int m1 = s == 0 ? n - 1 : s - 1;
      const int m2 = m1 == 0 ? n - 1 : m1 - 1;
      Nxx[s] = w * (((tx[s][1] * (sx[s][1] + sx[m1][2])) + (tx[m1][2] * (sx[m1][1] + sx[m2][2]))) + (Nx[s] * sx1));
      Nxy[s] = w * (((tx[s][1] * (sy[s][1] + sy[m1][2])) + (tx[m1][2] * (sy[m1][1] + sy[m2][2]))) + (Nx[s] * sy1));
      Nyy[s] = w * (((ty[s][1] * (sy[s][1] + sy[m1][2])) + (ty[m1][2] * (sy[m1][1] + sy[m2][2]))) + (Ny[s] * sy1));
    }
  } else {
    const double w = 1.0 / (double)(n - 1);
    double a = 0.0, b = 0.0;
    for (int t = 0; t < n - 1; ++t) a = a + tx[t][0];
    for (int t = 0; t < n - 1; ++t) b = b + ty[t][0];
    Nx[n] = w * a;  // A9a
    Ny[n] = w * b;
    for (int c = 0; c < n; ++c) {  // A9b
      if (c == 0) {
        Nx[c] = w * tx[0][1];
        Ny[c] = w * ty[0][1];
      } else if (c == n - 1) {
        Nx[c] = w * tx[n - 2][2];
        Ny[c] = w * ty[n - 2][2];
      } else {
        Nx[c] = w * (tx[c][1] + tx[c - 1][2]);
        Ny[c] = w * (ty[c][1] + ty[c - 1][2]);
      }
    }
    const double w2 = 1.0 / (double)(n - 2);
    for (int s = 0; s < n - 2; ++s) {  // A24a-c
      Nxx[n] = Nxx[n] + (w2 * (((sx[s][0] * Nx[n]) + (sx[s][1] * tx[s][0])) + (sx[s][2] * tx[s + 1][0])));
      Nxy[n] = Nxy[n] + (w2 * (((sy[s][0] * Nx[n]) + (sy[s][1] * tx[s][0])) + (sy[s][2] * tx[s + 1][0])));
      Nyy[n] = Nyy[n] + (w2 * (((sy[s][0] * Ny[n]) + (sy[s][1] * ty[s][0])) + (sy[s][2] * ty[s + 1][0])));
    }
    double sx1 = 0.0, sy1 = 0.0;
    for (int s = 0; s < n - 2; ++s) sx1 = sx1 + sx[s][0];
    for (int s = 0; s < n - 2; ++s) sy1 = sy1 + sy[s][0];
    for (int s = 0; s < n; ++s) {  // A24d-f with A25a-i; s is the 0-based neighbour
      double ax = 0.0, axy = 0.0, ay = 0.0, bx = 0.0, bxy = 0.0, by = 0.0, cx = 0.0, cxy = 0.0, cy = 0.0;
      if (s < n - 2) {
        ax = sx[s][1] * tx[s][1];
        axy = sy[s][1] * tx[s][1];
        ay = sy[s][1] * ty[s][1];
      }
      if (s > 0 && s < n - 1) {
        bx = (sx[s - 1][1] * tx[s - 1][2]) + (sx[s - 1][2] * tx[s][1]);
        bxy = (sy[s - 1][1] * tx[s - 1][2]) + (sy[s - 1][2] * tx[s][1]);
        by = (sy[s - 1][1] * ty[s - 1][2]) + (sy[s - 1][2] * ty[s][1]);
      }
      if (s > 1) {
        cx = sx[s - 2][2] * tx[s - 1][2];
        cxy = sy[s - 2][2] * tx[s - 1][2];
        cy = sy[s - 2][2] * ty[s - 1][2];
      }
      Nxx[s] = w2 * (((ax + bx) + cx) + (Nx[s] * sx1));
      Nxy[s] = w2 * (((axy + bxy) + cxy) + (Nx[s] * sy1));
      Nyy[s] = w2 * (((ay + by) + cy) + (Ny[s] * sy1));
    }
  }
}

namespace {

// Ordered queue with O(1) append, removal, top (last) and move-last-to-first.
struct LinkedQueue {
  std::vector<int> prev, next;
  std::vector<uint8_t> in;
  int head = -1, tail = -1, size = 0;
  explicit LinkedQueue(int n) : prev(n, -1), next(n, -1), in(n, 0) {}
  void push_back(int v) {
    prev[v] = tail;
    next[v] = -1;
    if (tail >= 0) next[tail] = v; else head = v;
    tail = v;
    in[v] = 1;
    ++size;
  }
  void remove(int v) {
    if (prev[v] >= 0) next[prev[v]] = next[v]; else head = next[v];
    if (next[v] >= 0) prev[next[v]] = prev[v]; else tail = prev[v];
    prev[v] = next[v] = -1;
    in[v] = 0;
    --size;
  }
  void rotate_last_to_front() {
    if (size < 2) return;
    const int v = tail;
    remove(v);
    prev[v] = -1;
    next[v] = head;
    prev[head] = v;
    head = v;
    in[v] = 1;
    ++size;
  }
};

struct Colouring {
  int nA, ncm;
  std::vector<int> deg;
  std::vector<int> L;      // row-major adjacency rows of width ncm, 0-based ids, -1 = empty
  LinkedQueue Q4, Q5;
  std::vector<int> S_vi;
  std::vector<int> S_L;    // snapshots of L rows at deletion
  int noofvert;
  int err = 0;

  Colouring(int n, int cm) : nA(n), ncm(cm), deg(n), L((size_t)n * cm, -1), Q4(n), Q5(n), noofvert(n) {
    S_vi.reserve(n);
    S_L.reserve((size_t)n * cm);
  }
  int *row(int v) { return &L[(size_t)v * ncm]; }

  // check(): keep v's queue membership consistent with its degree.
  void check(int v) {
    const int d = deg[v];
    if (d <= 4) {
      if (Q5.in[v]) Q5.remove(v);
      if (!Q4.in[v]) Q4.push_back(v);
    } else if (d == 5) {
      if (Q4.in[v]) Q4.remove(v);
      if (!Q5.in[v]) Q5.push_back(v);
    } else {
      if (Q4.in[v]) { err = UFE_BAD_MESH; return; }
      if (Q5.in[v]) Q5.remove(v);
    }
  }
  void remove_vertex(int v) {
    int *lv = row(v);
    for (int c = 0; c < deg[v]; ++c) {
      const int w = lv[c];
      int *lw = row(w);
      for (int c2 = 0; c2 < deg[w]; ++c2) {
        if (lw[c2] == v) {
          for (int k = c2; k < deg[w] - 1; ++k) lw[k] = lw[k + 1];
          lw[deg[w] - 1] = -1;
          --deg[w];
          check(w);
          break;
        }
      }
    }
    S_vi.push_back(v);
    S_L.insert(S_L.end(), lv, lv + ncm);
    if (deg[v] <= 4) Q4.remove(v);
    else if (deg[v] == 5) Q5.remove(v);
    else err = UFE_BAD_MESH;
    --noofvert;
  }
  bool adjacent(int x, int y) {
    const int *ly = row(y);
    for (int c = 0; c < deg[y]; ++c)
      if (ly[c] == x) return true;
    return false;
  }
  int reduce() {
    int64_t it = 0;
    while (noofvert > 5) {
      if (++it > 2 * (int64_t)nA) return UFE_BAD_MESH;  // "reduce got stuck"
      if (Q4.size > 0) {
        remove_vertex(Q4.tail);
        if (err) return err;
      } else {
        const int v = Q5.tail;
        const int *lv = row(v);
        bool found = false;
        for (int c1 = 0; c1 < deg[v] && !found; ++c1) {
          const int x = lv[c1];
          for (int c2 = c1 + 1; c2 < deg[v]; ++c2) {
            const int y = lv[c2];
            if (adjacent(x, y)) continue;
            if (deg[x] < ncm && deg[y] < ncm) { found = true; break; }
          }
        }
        // The reference deletes v and calls identify(x,y), which aborts unconditionally.
        if (found) return UFE_COLOUR_IDENTIFY;
        Q5.rotate_last_to_front();
      }
    }
    return UFE_OK;
  }
  int paint(std::vector<int> &colour) {
    // The (at most) five remaining vertices, in Q4 order, get colours 1..5.
    int k = 1;
    for (int v = Q4.head; v >= 0 && k <= 5; v = Q4.next[v]) colour[v] = k++;
    if (k != 6) return UFE_BAD_MESH;
    for (int s = (int)S_vi.size() - 1; s >= 0; --s) {
      const int v = S_vi[s];
      const int *lv = &S_L[(size_t)s * ncm];
      int used = 0;
      for (int c = 0; c < ncm; ++c) {
        const int u = lv[c];
        if (u < 0) break;
        if (colour[u] != 0) used |= 1 << (colour[u] - 1);
      }
      if (used == 31) return UFE_BAD_MESH;
      for (int c = 1; c <= 5; ++c)
        if (!(used & (1 << (c - 1)))) { colour[v] = c; break; }
    }
    return UFE_OK;
  }
};

}  // namespace

int aaac_build(const ufe_base_mesh *b, ufe_aaac_mesh *o, std::string *msg) {
  const int nV = b->nV, ncm = b->nC_mem, nT = b->nTri;
  if (nV < 5 || ncm < 3 || ncm > kMaxDeg - 1 || nT < 4) { *msg = "bad base mesh sizes"; return UFE_BAD_ARG; }
  const int nAc = nV + nT - 1;
  const int nA = nV + nAc;
  if (o->nAc != nAc || o->nVAaAc != nA) { *msg = "output nAc/nVAaAc must be nV+nTri-1 / nV+nAc"; return UFE_BAD_ARG; }
  const double *V = b->V;
  auto X = [&](int v) { return V[v]; };
  auto Y = [&](int v) { return V[v + (int64_t)nV]; };
  auto C = [&](int v, int c) { return b->C[v + (int64_t)c * nV] - 1; };
  auto nC = [&](int v) { return b->nC[v]; };
  auto edge = b->edge_index;

  // Aa neighbour functions (get_neighbour_functions, vertex part).
  if (o->Nx) {
    double qx[kMaxDeg], qy[kMaxDeg], f[5][kMaxDeg + 1];
    for (int v = 0; v < nV; ++v) {
      const int n = nC(v);
      for (int c = 0; c < n; ++c) { qx[c] = X(C(v, c)); qy[c] = Y(C(v, c)); }
      neighbour_functions(X(v), Y(v), n, qx, qy, edge[v] > 0, f[0], f[1], f[2], f[3], f[4]);
      double *dst[5] = {o->Nx, o->Ny, o->Nxx, o->Nxy, o->Nyy};
      for (int q = 0; q < 5; ++q)
        for (int c = 0; c <= ncm; ++c) dst[q][v + (int64_t)c * nV] = c <= n ? f[q][c] : 0.0;
    }
  }

  // Ac numbering: visit vi = 1..nV, ci = 1..nC(vi), skipping connections already numbered
  // from the other side.
  std::vector<int> iAci((size_t)nV * ncm, -1);  // 0-based Ac id, row-major (v,c)
  std::vector<int> Aci((size_t)nAc * 4, 0);     // 0-based vertex ids, row-major (ac,k)
  std::vector<double> NxAc((size_t)nAc * 4), NyAc((size_t)nAc * 4), NoAc((size_t)nAc * 4), NpAc(nAc);
  int ac = 0, vl = 0, vr = 0;
  for (int vi = 0; vi < nV; ++vi) {
    for (int ci = 0; ci < nC(vi); ++ci) {
      if (iAci[(size_t)vi * ncm + ci] >= 0) continue;
      const int vj = C(vi, ci);
      if (ac >= nAc) { *msg = "more connections than nV+nTri-1"; return UFE_BAD_MESH; }
      iAci[(size_t)vi * ncm + ci] = ac;
      for (int cj = 0; cj < nC(vj); ++cj)
        if (C(vj, cj) == vi) { iAci[(size_t)vj * ncm + cj] = ac; break; }
      const bool bseg = boundary_segment(edge, vi, vj);
      // Third vertices of the triangles left (vi,vj,vl) and right (vj,vi,vr) of the edge.
      for (int t = 0; t < b->niTri[vi]; ++t) {
        const int ti = b->iTri[vi + (int64_t)t * nV] - 1;
        for (int k = 0; k < 3; ++k) {
          const int a0 = b->Tri[ti + (int64_t)k * nT] - 1;
          const int a1 = b->Tri[ti + (int64_t)((k + 1) % 3) * nT] - 1;
          const int a2 = b->Tri[ti + (int64_t)((k + 2) % 3) * nT] - 1;
          if (!bseg) {
            if (a0 == vi && a1 == vj) vl = a2;
            else if (a0 == vj && a1 == vi) vr = a2;
          } else if ((a0 == vi && a1 == vj) || (a0 == vj && a1 == vi)) {
            vl = a2;
          }
        }
      }
      int *ai = &Aci[(size_t)ac * 4];
      double nx[4], ny[4];
      const double dyl = Y(vl) - Y(vj), dyi = Y(vi) - Y(vl), dyj = Y(vj) - Y(vi);
      const double dxl = X(vj) - X(vl), dxi = X(vl) - X(vi), dxj = X(vi) - X(vj);
      const double nzl = ((X(vj) - X(vi)) * (Y(vl) - Y(vi))) - ((Y(vj) - Y(vi)) * (X(vl) - X(vi)));
      if (!bseg) {
        ai[0] = vi; ai[1] = vj; ai[2] = vl; ai[3] = vr;
        const double nzr = ((X(vr) - X(vi)) * (Y(vj) - Y(vi))) - ((Y(vr) - Y(vi)) * (X(vj) - X(vi)));
        const double lx[4] = {dyl, dyi, dyj, 0.0}, ly[4] = {dxl, dxi, dxj, 0.0};
        const double rx[4] = {Y(vj) - Y(vr), Y(vr) - Y(vi), 0.0, Y(vi) - Y(vj)};
        const double ry[4] = {X(vr) - X(vj), X(vi) - X(vr), 0.0, X(vj) - X(vi)};
        for (int k = 0; k < 4; ++k) {
          nx[k] = -((lx[k] / nzl) + (rx[k] / nzr)) / 2.0;
          ny[k] = -((ly[k] / nzl) + (ry[k] / nzr)) / 2.0;
        }
      } else {
        ai[0] = vi; ai[1] = vj; ai[2] = vl; ai[3] = 0;  // 4th entry "1" in the reference
        const double lx[4] = {dyl, dyi, dyj, 0.0}, ly[4] = {dxl, dxi, dxj, 0.0};
        for (int k = 0; k < 4; ++k) {
          nx[k] = -lx[k] / nzl;
          ny[k] = -ly[k] / nzl;
        }
      }
      const double ux = X(vj) - X(vi), uy = Y(vj) - Y(vi);
      const double u = std::sqrt(ux * ux + uy * uy);
      for (int k = 0; k < 4; ++k) {
        NxAc[(size_t)ac * 4 + k] = nx[k];
        NyAc[(size_t)ac * 4 + k] = ny[k];
        NoAc[(size_t)ac * 4 + k] = ((ny[k] * ux) - (nx[k] * uy)) / u;
      }
      NpAc[ac] = 1.0 / u;
      ++ac;
    }
  }
  if (ac != nAc) { *msg = "connection count differs from nV+nTri-1 (not a triangulated disc)"; return UFE_BAD_MESH; }

  // Ac edge indices (find_Ac_edge_indices): both ends on the same side of the square.
  std::vector<int> eAc(nAc);
  for (int a = 0; a < nAc; ++a) {
    const int ei = edge[Aci[(size_t)a * 4]], ej = edge[Aci[(size_t)a * 4 + 1]];
    auto on = [](int e, int side) {  // side 1,3,5,7 with its two corners
      const int lo = side == 1 ? 8 : side - 1;
      return e == lo || e == side || e == side + 1;
    };
    eAc[a] = (on(ei, 1) && on(ej, 1)) ? 1 : (on(ei, 3) && on(ej, 3)) ? 3 : (on(ei, 5) && on(ej, 5)) ? 5
             : (on(ei, 7) && on(ej, 7)) ? 7 : 0;
  }

  // Combined AaAc connectivity (0-based ids: Aa vertex v -> v, Ac vertex a -> nV + a).
  std::vector<int> nCA(nA);
  std::vector<int> CA((size_t)nA * ncm, -1);
  for (int v = 0; v < nV; ++v) {
    nCA[v] = nC(v);
    for (int c = 0; c < nC(v); ++c) CA[(size_t)v * ncm + c] = iAci[(size_t)v * ncm + c] + nV;
  }
  auto ac_between = [&](int centre, int other) {  // Ac id of connection centre-other; last match
    int found = -1;
    for (int c = 0; c < nC(centre); ++c)
      if (C(centre, c) == other) found = iAci[(size_t)centre * ncm + c];
    return found;
  };
  for (int a = 0; a < nAc; ++a) {
    const int r = nV + a;
    int vi = Aci[(size_t)a * 4], vj = Aci[(size_t)a * 4 + 1];
    int *row = &CA[(size_t)r * ncm];
    if (eAc[a] > 0) {
      bool sw = false;
      switch (eAc[a]) {
        case 1: sw = X(vi) > X(vj); break;
        case 3: sw = Y(vi) < Y(vj); break;
        case 5: sw = X(vi) < X(vj); break;
        case 7: sw = Y(vi) > Y(vj); break;
      }
      if (sw) { const int t = vi; vi = vj; vj = t; }
      const int vk = Aci[(size_t)a * 4 + 2];
      const int a1 = ac_between(vk, vi), a2 = ac_between(vk, vj);
      if (a1 < 0 || a2 < 0) { *msg = "couldnt find Ac vertex"; return UFE_BAD_MESH; }
      nCA[r] = 4;
      row[0] = vi; row[1] = a1 + nV; row[2] = a2 + nV; row[3] = vj;
    } else {
      const int l = Aci[(size_t)a * 4 + 2], rr = Aci[(size_t)a * 4 + 3];
      const int a1 = ac_between(rr, vi), a2 = ac_between(rr, vj);
      const int a3 = ac_between(l, vj), a4 = ac_between(l, vi);
      if (a1 < 0 || a2 < 0 || a3 < 0 || a4 < 0) { *msg = "couldnt find Ac vertex"; return UFE_BAD_MESH; }
      nCA[r] = 6;
      row[0] = vi; row[1] = a1 + nV; row[2] = a2 + nV; row[3] = vj; row[4] = a3 + nV; row[5] = a4 + nV;
    }
  }

  // Coordinates of the combined mesh and its neighbour functions.
  auto AX = [&](int r) { return r < nV ? X(r) : (X(Aci[(size_t)(r - nV) * 4]) + X(Aci[(size_t)(r - nV) * 4 + 1])) / 2.0; };
  auto AY = [&](int r) { return r < nV ? Y(r) : (Y(Aci[(size_t)(r - nV) * 4]) + Y(Aci[(size_t)(r - nV) * 4 + 1])) / 2.0; };
  {
    double qx[kMaxDeg], qy[kMaxDeg], f[5][kMaxDeg + 1];
    double *dst[5] = {o->Nx_AaAc, o->Ny_AaAc, o->Nxx_AaAc, o->Nxy_AaAc, o->Nyy_AaAc};
    for (int r = 0; r < nA; ++r) {
      const int n = nCA[r];
      for (int c = 0; c < n; ++c) { qx[c] = AX(CA[(size_t)r * ncm + c]); qy[c] = AY(CA[(size_t)r * ncm + c]); }
      const bool is_edge = r < nV ? edge[r] > 0 : eAc[r - nV] > 0;
      neighbour_functions(AX(r), AY(r), n, qx, qy, is_edge, f[0], f[1], f[2], f[3], f[4]);
      for (int q = 0; q < 5; ++q)
        if (dst[q])
          for (int c = 0; c <= ncm; ++c) dst[q][r + (int64_t)c * nA] = c <= n ? f[q][c] : 0.0;
    }
  }

  // Write the Fortran-layout outputs.
  for (int v = 0; v < nV; ++v)
    for (int c = 0; c < ncm; ++c) o->iAci[v + (int64_t)c * nV] = c < nC(v) ? iAci[(size_t)v * ncm + c] + 1 : 0;
  for (int a = 0; a < nAc; ++a) {
    for (int k = 0; k < 4; ++k) {
      o->Aci[a + (int64_t)k * nAc] = Aci[(size_t)a * 4 + k] + 1;
      if (o->Nx_Ac) o->Nx_Ac[a + (int64_t)k * nAc] = NxAc[(size_t)a * 4 + k];
      if (o->Ny_Ac) o->Ny_Ac[a + (int64_t)k * nAc] = NyAc[(size_t)a * 4 + k];
      if (o->No_Ac) o->No_Ac[a + (int64_t)k * nAc] = NoAc[(size_t)a * 4 + k];
    }
    if (o->Np_Ac) o->Np_Ac[a] = NpAc[a];
    if (o->VAc) { o->VAc[a] = AX(nV + a); o->VAc[a + (int64_t)nAc] = AY(nV + a); }
    o->edge_index_Ac[a] = eAc[a];
  }
  for (int r = 0; r < nA; ++r) {
    o->nCAaAc[r] = nCA[r];
    for (int c = 0; c < ncm; ++c) o->CAaAc[r + (int64_t)c * nA] = CA[(size_t)r * ncm + c] + 1;  // -1 -> 0
    if (o->VAaAc) { o->VAaAc[r] = AX(r); o->VAaAc[r + (int64_t)nA] = AY(r); }
  }

  // Five-colouring.
  if (o->colour) {
    Colouring col(nA, ncm);
    for (int r = 0; r < nA; ++r) {
      col.deg[r] = nCA[r];
      std::memcpy(col.row(r), &CA[(size_t)r * ncm], sizeof(int) * ncm);
    }
    for (int r = 0; r < nA; ++r) {
      if (col.deg[r] <= 4) col.Q4.push_back(r);
      else if (col.deg[r] == 5) col.Q5.push_back(r);
    }
    int rc = col.reduce();
    if (rc != UFE_OK) {
      *msg = rc == UFE_COLOUR_IDENTIFY ? "five-colouring reached identify (reference aborts there)"
                                       : "five-colouring reduction failed";
      return rc;
    }
    std::vector<int> colour(nA, 0);
    rc = col.paint(colour);
    if (rc != UFE_OK) { *msg = "five-colouring paint failed"; return rc; }
    for (int r = 0; r < nA; ++r)  // check_solution
      for (int c = 0; c < nCA[r]; ++c)
        if (colour[r] == 0 || colour[r] == colour[CA[(size_t)r * ncm + c]]) {
          *msg = "the resulting five-colouring is invalid";
          return UFE_BAD_MESH;
        }
    int cnt[5] = {0, 0, 0, 0, 0};
    std::memset(o->colour_vi, 0, sizeof(int32_t) * (size_t)nA * 5);
    for (int r = 0; r < nA; ++r) {
      const int c = colour[r] - 1;
      o->colour[r] = colour[r];
      o->colour_vi[cnt[c] + (int64_t)c * nA] = r + 1;
      ++cnt[c];
    }
    for (int c = 0; c < 5; ++c) o->colour_nV[c] = cnt[c];
  }
  return UFE_OK;
}

}  // namespace ufe
