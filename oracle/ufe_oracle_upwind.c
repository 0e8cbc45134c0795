/*
 * CPU oracle, upwind derivatives for thermodynamics -- TEST INFRASTRUCTURE ONLY (see ufe_oracle.h).
 *
 * Literal FP64 restatements of
 *   get_upwind_derivative_vertex_3D   mesh_derivatives_module.f90:434-483
 *   get_mesh_derivatives_vertex_3D    mesh_derivatives_module.f90:372-392 (the no-wind case)
 *   is_in_triangle                    mesh_help_functions_module.f90:646-672
 *   the triangle functions NxTri/NyTri of get_neighbour_functions, mesh_derivatives_module.f90:30-47
 *   the vertex resolution mesh%R      mesh_help_functions_module.f90:195-211
 */
#include <math.h>
#include <stddef.h>

#include "ufe_oracle.h"

#define A1(p, i) ((p)[(size_t)(i) - 1])
#define A2(p, ld, i, j) ((p)[(size_t)((i) - 1) + (size_t)((j) - 1) * (size_t)(ld)])

void or_triangle_functions(const or_base *b, double *NxTri, double *NyTri) {
  const int nT = b->nTri, nV = b->nV;
  for (int ti = 1; ti <= nT; ti++) {
    const int va = A2(b->Tri, nT, ti, 1), vb = A2(b->Tri, nT, ti, 2), vc = A2(b->Tri, nT, ti, 3);
    const double ax = A2(b->V, nV, va, 1), ay = A2(b->V, nV, va, 2);
    const double bx = A2(b->V, nV, vb, 1), by = A2(b->V, nV, vb, 2);
    const double cx = A2(b->V, nV, vc, 1), cy = A2(b->V, nV, vc, 2);
    const double D = ax * (by - cy) + bx * (cy - ay) + cx * (ay - by);
    A2(NxTri, nT, ti, 1) = (by - cy) / D;
    A2(NxTri, nT, ti, 2) = (cy - ay) / D;
    A2(NxTri, nT, ti, 3) = (ay - by) / D;
    A2(NyTri, nT, ti, 1) = (cx - bx) / D;
    A2(NyTri, nT, ti, 2) = (ax - cx) / D;
    A2(NyTri, nT, ti, 3) = (bx - ax) / D;
  }
}

void or_vertex_resolution(const or_base *b, double domain_width, double *R) {
  const int nV = b->nV;
  for (int vi = 1; vi <= nV; vi++) A1(R, vi) = domain_width;
  for (int vi = 1; vi <= nV; vi++)
    for (int ci = 1; ci <= A1(b->nC, vi); ci++) {
      const int vj = A2(b->C, nV, vi, ci);
      const double dx = A2(b->V, nV, vj, 1) - A2(b->V, nV, vi, 1);
      const double dy = A2(b->V, nV, vj, 2) - A2(b->V, nV, vi, 2);
      const double r = sqrt(dx * dx + dy * dy);
      if (r < A1(R, vi)) A1(R, vi) = r;
    }
}

static int is_in_triangle(double pax, double pay, double pbx, double pby, double pcx, double pcy, double px,
                          double py) {
  const double tol = 1E-8;
  const double as_x = px - pax, as_y = py - pay;
  const double s1 = ((pbx - pax) * as_y - (pby - pay) * as_x);
  const double s2 = ((pcx - pax) * as_y - (pcy - pay) * as_x);
  const double s3 = ((pcx - pbx) * (py - pby) - (pcy - pby) * (px - pbx));
  return s1 > -tol && s2 < tol && s3 > -tol;
}

long long or_upwind_derivatives_3d(const or_base *b, const or_aaac *m, int nZ, const double *R, const double *NxTri,
                                   const double *NyTri, const double *U, const double *V, const double *d,
                                   double *ddx, double *ddy) {
  const int nV = b->nV, nT = b->nTri;
  long long missing = 0;
  for (int k = 1; k <= nZ; k++)
    for (int vi = 1; vi <= nV; vi++) {
      const double u = A2(U, nV, vi, k), v = A2(V, nV, vi, k);
      double dx = 0.0, dy = 0.0;
      if (fabs(u) < 1E-10 && fabs(v) < 1E-10) {
        const int n = A1(b->nC, vi);
        dx = A2(m->Nx, nV, vi, n + 1) * A2(d, nV, vi, k);
        dy = A2(m->Ny, nV, vi, n + 1) * A2(d, nV, vi, k);
        for (int ci = 1; ci <= n; ci++) {
          const int vc = A2(b->C, nV, vi, ci);
          dx = dx + A2(m->Nx, nV, vi, ci) * A2(d, nV, vc, k);
          dy = dy + A2(m->Ny, nV, vi, ci) * A2(d, nV, vc, k);
        }
      } else {
        const double s = 4.0 * sqrt(u * u + v * v);
        const double px = A2(b->V, nV, vi, 1) - u * A1(R, vi) / s;
        const double py = A2(b->V, nV, vi, 2) - v * A1(R, vi) / s;
        int tup = 0;
        for (int iti = 1; iti <= A1(b->niTri, vi); iti++) {
          const int ti = A2(b->iTri, nV, vi, iti);
          const int va = A2(b->Tri, nT, ti, 1), vb = A2(b->Tri, nT, ti, 2), vc = A2(b->Tri, nT, ti, 3);
          if (is_in_triangle(A2(b->V, nV, va, 1), A2(b->V, nV, va, 2), A2(b->V, nV, vb, 1), A2(b->V, nV, vb, 2),
                             A2(b->V, nV, vc, 1), A2(b->V, nV, vc, 2), px, py)) {
            tup = ti;
            break;
          }
        }
        if (tup == 0) {
          /* the reference reports the vertex and reads row 0 of NxTri, outside the array */
          missing++;
        } else {
          const int va = A2(b->Tri, nT, tup, 1), vb = A2(b->Tri, nT, tup, 2), vc = A2(b->Tri, nT, tup, 3);
          dx = A2(NxTri, nT, tup, 1) * A2(d, nV, va, k) + A2(NxTri, nT, tup, 2) * A2(d, nV, vb, k) +
               A2(NxTri, nT, tup, 3) * A2(d, nV, vc, k);
          dy = A2(NyTri, nT, tup, 1) * A2(d, nV, va, k) + A2(NyTri, nT, tup, 2) * A2(d, nV, vb, k) +
               A2(NyTri, nT, tup, 3) * A2(d, nV, vc, k);
        }
      }
      A2(ddx, nV, vi, k) = dx;
      A2(ddy, nV, vi, k) = dy;
    }
  return missing;
}
