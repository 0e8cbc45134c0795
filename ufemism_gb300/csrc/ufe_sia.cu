// SIA velocities on the staggered (Ac) mesh: solve_SIA, ice_dynamics_module.f90:240-314,
// with vertical_integrate / vertical_average (zeta_module.f90:33-85) and map_Ac_to_Aa
// (mesh_ArakawaC_module.f90:770-791).
//
// One thread per Ac edge, columns of the (nAc, nZ) arrays read and written level by level
// (column-major, so each level is a coalesced row of the warp). The edge kernel is a pure
// stream (A_flow_Ac in, D_SIA_3D_Ac out, about 2 * 8 * nZ bytes per edge); the Aa average is
// a small gather over iAci. Built with --fmad=false: every product and sum rounds as in the
// reference.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "ufe_internal.h"

namespace ufe {

constexpr int kMaxZ = 64;

struct SiaWork {
  int nV = 0, nAc = 0, nZ = 0;
  double *in = nullptr;    // H, sx, sy, sp, so (5 nAc) + A_flow (nAc nZ)
  int *mask = nullptr;     // nAc
  double *out = nullptr;   // D3 (nAc nZ), D, Ux, Uy, Up, Uo (5 nAc), U, V, D Aa (3 nV)
  double *zc = nullptr;    // zeta (nZ), zeta^3 (nZ)
  bool solved = false;
};

void sia_free(SiaWork *w) {
  if (!w) return;
  if (w->in) cudaFree(w->in);
  if (w->mask) cudaFree(w->mask);
  if (w->out) cudaFree(w->out);
  if (w->zc) cudaFree(w->zc);
  delete w;
}

template <int NZ>
__global__ void __launch_bounds__(256) k_sia_edges(int nAc, int nZ_rt, const int *__restrict__ mask,
                                                   const double *__restrict__ H, const double *__restrict__ sx,
                                                   const double *__restrict__ sy, const double *__restrict__ sp,
                                                   const double *__restrict__ so, const double *__restrict__ A,
                                                   const double *__restrict__ zeta, const double *__restrict__ zeta3,
                                                   double m_enh, double *__restrict__ D3, double *__restrict__ D,
                                                   double *__restrict__ Ux, double *__restrict__ Uy,
                                                   double *__restrict__ Up, double *__restrict__ Uo) {
  const int nZ = NZ > 0 ? NZ : nZ_rt;
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nAc) return;
  const size_t ld = (size_t)nAc;
  const double cutoff = -1e5;
  double d3[NZ > 0 ? NZ : kMaxZ];
  if (mask[a] == 1) {
    const double h = H[a];
    const double p = sp[a], o = so[a];
    // (rho g H)^n * (dHs_dp^2 + dHs_do^2)^((n-1)/2), n = 3: the second power is 1.
    const double D0 = pow((kIceDensity * kGrav) * h, 3.0) * (p * p + o * o);
    // vertical_integrate( m_enh_sia * A_flow * zeta^n ), from the base upwards
    double f_hi = (m_enh * A[a + (size_t)(nZ - 1) * ld]) * zeta3[nZ - 1];
    double acc = 0.0;
    d3[nZ - 1] = 0.0;
#pragma unroll
    for (int k = nZ - 2; k >= 0; --k) {
      const double f_lo = (m_enh * A[a + (size_t)k * ld]) * zeta3[k];
      acc = acc - (0.5 * (f_hi + f_lo)) * (zeta[k + 1] - zeta[k]);
      d3[k] = acc;
      f_hi = f_lo;
    }
    const double h2 = 2.0 * h;
#pragma unroll
    for (int k = 0; k < nZ; ++k) {
      double v = D0 * (h2 * d3[k]);
      if (v < cutoff) v = cutoff;
      d3[k] = v;
      if (D3) D3[a + (size_t)k * ld] = v;
    }
    // vertical_average
    double avg = 0.0;
#pragma unroll
    for (int k = 0; k < nZ - 1; ++k) avg = avg + (0.5 * (d3[k + 1] + d3[k])) * (zeta[k + 1] - zeta[k]);
    D[a] = h * avg;
    Ux[a] = avg * sx[a];
    Uy[a] = avg * sy[a];
    Up[a] = avg * p;
    Uo[a] = avg * o;
  } else {
    if (D3)
      for (int k = 0; k < nZ; ++k) D3[a + (size_t)k * ld] = 0.0;
    D[a] = 0.0; Ux[a] = 0.0; Uy[a] = 0.0; Up[a] = 0.0; Uo[a] = 0.0;
  }
}

// map_Ac_to_Aa for three fields: d_Aa(vi) = sum_ci d_Ac(iAci(vi,ci)) / nC(vi), in ci order.
__global__ void k_ac_to_aa3(int nV, const int *__restrict__ nC, const int *__restrict__ iAci,
                            const double *__restrict__ a0, const double *__restrict__ a1,
                            const double *__restrict__ a2, double *__restrict__ b0,
                            double *__restrict__ b1, double *__restrict__ b2) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nV) return;
  const int n = nC[v];
  const double dn = (double)n;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int c = 0; c < n; ++c) {
    const int a = iAci[v + (size_t)c * nV];
    s0 = s0 + a0[a] / dn;
    s1 = s1 + a1[a] / dn;
    s2 = s2 + a2[a] / dn;
  }
  b0[v] = s0;
  b1[v] = s1;
  b2[v] = s2;
}

}  // namespace ufe

using namespace ufe;

namespace ufe {
// Up_SIA_Ac of the last ufe_sia_solve on this handle, on the device, or null.
const double *sia_device_Up(ufe_mesh_h h) {
  const SiaWork *w = h->sia;
  if (!w || !w->solved) return nullptr;
  const size_t na = w->nAc;
  return w->out + na * w->nZ + 3 * na;
}
}  // namespace ufe

namespace ufe {
// ufe_sia_solve; with fields_on_device the mask and the five Ac fields of `in` are device
// arrays of this device (the device geometry preparation), and with A_on_device A_flow_Ac is
// too (the device physical properties); otherwise A_flow_Ac is a host array.
int sia_solve_impl(ufe_mesh_h h, const ufe_params *p, const ufe_sia_in *in, ufe_sia_out *out, bool fields_on_device,
                   bool A_on_device) {
  if (!h || !p || !in || !out) { set_error("ufe_sia_solve: null argument"); return UFE_BAD_ARG; }
  if (!in->mask_sheet_Ac || !in->Hi_Ac || !in->dHs_dx_Ac || !in->dHs_dy_Ac || !in->dHs_dp_Ac ||
      !in->dHs_do_Ac || !in->A_flow_Ac || !p->zeta) {
    set_error("ufe_sia_solve: missing input array");
    return UFE_BAD_ARG;
  }
  if (p->nZ < 2 || p->nZ > kMaxZ) { set_error("ufe_sia_solve: nZ must be in [2, 64]"); return UFE_BAD_ARG; }
  const DevMesh &m = h->m;
  const int nV = m.nV, nAc = m.nAc, nZ = p->nZ;
  cudaStream_t s = h->stream;
  int rc = UFE_OK;
  if (h->sia && h->sia->nZ != nZ) { sia_free(h->sia); h->sia = nullptr; }
  if (!h->sia) {
    SiaWork *w = new SiaWork();
    w->nV = nV; w->nAc = nAc; w->nZ = nZ;
    rc = cuda_status(cudaMalloc(&w->in, ((size_t)5 + nZ) * nAc * sizeof(double)), "sia in");
    if (!rc) rc = cuda_status(cudaMalloc(&w->mask, (size_t)nAc * sizeof(int)), "sia mask");
    if (!rc) rc = cuda_status(cudaMalloc(&w->out, (((size_t)5 + nZ) * nAc + 3 * (size_t)nV) * sizeof(double)), "sia out");
    if (!rc) rc = cuda_status(cudaMalloc(&w->zc, 2 * (size_t)nZ * sizeof(double)), "sia zeta");
    if (rc) { sia_free(w); return rc; }
    h->sia = w;
  }
  SiaWork *w = h->sia;
  // zeta and zeta**n_flow (n = 3), the latter evaluated once on the host.
  std::vector<double> zc(2 * (size_t)nZ);
  for (int k = 0; k < nZ; ++k) { zc[k] = p->zeta[k]; zc[nZ + k] = std::pow(p->zeta[k], 3.0); }
  const size_t na = nAc;
  double *H = w->in, *sx = H + na, *sy = sx + na, *sp = sy + na, *so = sp + na, *A = so + na;
  rc = cuda_status(cudaMemcpyAsync(w->zc, zc.data(), zc.size() * sizeof(double), cudaMemcpyHostToDevice, s), "H2D zeta");
  const cudaMemcpyKind kin = fields_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (!rc) rc = cuda_status(cudaMemcpyAsync(w->mask, in->mask_sheet_Ac, na * sizeof(int), kin, s), "sia input");
  const double *src[5] = {in->Hi_Ac, in->dHs_dx_Ac, in->dHs_dy_Ac, in->dHs_dp_Ac, in->dHs_do_Ac};
  for (int k = 0; k < 5 && !rc; ++k)
    rc = cuda_status(cudaMemcpyAsync(w->in + k * na, src[k], na * sizeof(double), kin, s), "sia input");
  if (!rc)
    rc = cuda_status(cudaMemcpyAsync(A, in->A_flow_Ac, na * nZ * sizeof(double),
                                     A_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s), "A_flow input");
  double *D3 = w->out, *D = D3 + na * nZ, *Ux = D + na, *Uy = Ux + na, *Up = Uy + na, *Uo = Up + na;
  double *Ua = Uo + na, *Va = Ua + nV, *Da = Va + nV;
  if (!rc) {
    const unsigned g = (unsigned)((nAc + 255) / 256);
    if (nZ == 15)
      k_sia_edges<15><<<g, 256, 0, s>>>(nAc, nZ, w->mask, H, sx, sy, sp, so, A, w->zc, w->zc + nZ, p->m_enh_sia, D3, D, Ux, Uy, Up, Uo);
    else
      k_sia_edges<0><<<g, 256, 0, s>>>(nAc, nZ, w->mask, H, sx, sy, sp, so, A, w->zc, w->zc + nZ, p->m_enh_sia, D3, D, Ux, Uy, Up, Uo);
    rc = cuda_status(cudaGetLastError(), "k_sia_edges");
  }
  if (!rc) {
    k_ac_to_aa3<<<(unsigned)((nV + 255) / 256), 256, 0, s>>>(nV, m.nC, m.iAci, Ux, Uy, D, Ua, Va, Da);
    rc = cuda_status(cudaGetLastError(), "k_ac_to_aa3");
  }
  auto back = [&](double *dst, const double *srcd, size_t n) {
    if (!dst || rc) return;
    rc = cuda_status(cudaMemcpyAsync(dst, srcd, n * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
  };
  back(out->D_SIA_3D_Ac, D3, na * nZ);
  back(out->D_SIA_Ac, D, na);
  back(out->Ux_SIA_Ac, Ux, na);
  back(out->Uy_SIA_Ac, Uy, na);
  back(out->Up_SIA_Ac, Up, na);
  back(out->Uo_SIA_Ac, Uo, na);
  back(out->U_SIA, Ua, nV);
  back(out->V_SIA, Va, nV);
  back(out->D_SIA, Da, nV);
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "sia solve");
  w->solved = rc == UFE_OK;
  return rc;
}
}  // namespace ufe

extern "C" int ufe_sia_solve(ufe_mesh_h h, const ufe_params *p, const ufe_sia_in *in, ufe_sia_out *out) {
  return sia_solve_impl(h, p, in, out, false);
}

// ---------------------------------------------------------------------------------------
// solve_SIA without allocation: device-resident inputs and outputs, intermediates in a
// fixed scratch array of this translation unit.
//
// Who needs it: a model that keeps its ice state on the device and reserves its device
// memory up front (its own pool sized to the HBM it wants), and a time loop that must not
// stall: cudaMalloc and cudaFree synchronise the whole device, and the per-handle buffers of
// ufe_sia_solve are (re)allocated on the first call and whenever nZ changes. This entry
// point calls neither; its only device memory beyond the caller's arrays is the scratch
// below, which exists from the moment the module is loaded.
// ---------------------------------------------------------------------------------------
namespace ufe {
namespace {

constexpr int kNoAllocMaxAc = UFE_SIA_NOALLOC_MAX_AC;
constexpr int kNoAllocMaxDevices = 64;
// Layout: zeta (kMaxZ), zeta^3 (kMaxZ), then D, Ux, Uy, Up, Uo on the Ac edges (kNoAllocMaxAc
// each): 2 * 64 + 5 * 262,144 doubles = 10 MiB + 1 KiB.
constexpr size_t kNoAllocScratch = 2 * (size_t)kMaxZ + 5 * (size_t)kNoAllocMaxAc;
static __device__ __align__(256) double g_sia_scratch[kNoAllocScratch];

std::mutex g_scratch_mutex;
double *g_scratch_ptr[kNoAllocMaxDevices] = {};

// Address of the scratch on the current device, looked up once per device.
int scratch_address(int device, double **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[device]) {
    double *p = nullptr;
    const int rc = cuda_status(cudaGetSymbolAddress((void **)&p, g_sia_scratch), "cudaGetSymbolAddress(scratch)");
    if (rc) return rc;
    g_scratch_ptr[device] = p;
  }
  *out = g_scratch_ptr[device];
  return UFE_OK;
}

// The kernels dereference every array given, so each must be device memory of this device
// (or managed memory); a host pointer is rejected here instead of faulting there.
bool on_device(const void *ptr, int device) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) { cudaGetLastError(); return false; }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == device;
}

}  // namespace
}  // namespace ufe

extern "C" int ufe_sia_solve_noalloc(ufe_mesh_h h, const ufe_params *p, const ufe_sia_in *in, ufe_sia_out *out) {
  if (!h || !p || !in || !out) { set_error("ufe_sia_solve_noalloc: null argument"); return UFE_BAD_ARG; }
  const char *who = "ufe_sia_solve_noalloc";
  if (!in->mask_sheet_Ac || !in->Hi_Ac || !in->dHs_dx_Ac || !in->dHs_dy_Ac || !in->dHs_dp_Ac ||
      !in->dHs_do_Ac || !in->A_flow_Ac || !p->zeta) {
    set_error(std::string(who) + ": missing input array");
    return UFE_BAD_ARG;
  }
  if (p->nZ < 2 || p->nZ > kMaxZ) { set_error(std::string(who) + ": nZ must be in [2, 64]"); return UFE_BAD_ARG; }
  const DevMesh &m = h->m;
  const int nV = m.nV, nAc = m.nAc, nZ = p->nZ;
  if (nAc > kNoAllocMaxAc) {
    char buf[192];
    std::snprintf(buf, sizeof buf, "%s: the mesh has %d Ac edges; the fixed scratch holds at most %d", who, nAc,
                  kNoAllocMaxAc);
    set_error(buf);
    return UFE_BAD_ARG;
  }
  if (!out->U_SIA != !out->V_SIA || !out->U_SIA != !out->D_SIA) {
    set_error(std::string(who) + ": U_SIA, V_SIA and D_SIA are given together or not at all");
    return UFE_BAD_ARG;
  }
  int dev = -1;
  int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev != h->device || dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error(std::string(who) + ": the mesh's device must be the current device");
    return UFE_BAD_ARG;
  }
  const void *ins[7] = {in->mask_sheet_Ac, in->Hi_Ac, in->dHs_dx_Ac, in->dHs_dy_Ac, in->dHs_dp_Ac, in->dHs_do_Ac,
                        in->A_flow_Ac};
  const void *outs[9] = {out->D_SIA_3D_Ac, out->D_SIA_Ac, out->Ux_SIA_Ac, out->Uy_SIA_Ac, out->Up_SIA_Ac,
                         out->Uo_SIA_Ac, out->U_SIA, out->V_SIA, out->D_SIA};
  for (const void *q : ins)
    if (!on_device(q, dev)) { set_error(std::string(who) + ": an input array is not device memory of the mesh's device"); return UFE_BAD_ARG; }
  for (const void *q : outs)
    if (q && !on_device(q, dev)) { set_error(std::string(who) + ": an output array is not device memory of the mesh's device"); return UFE_BAD_ARG; }
  double *scratch = nullptr;
  rc = scratch_address(dev, &scratch);
  if (rc) return rc;
  // This call's results live only in the caller's arrays. An earlier ufe_sia_solve's
  // velocities on the handle are now out of date, so they are no longer offered to a
  // thickness update that is given no Up_SIA_Ac (it returns UFE_BAD_ARG instead).
  if (h->sia) h->sia->solved = false;
  cudaStream_t s = h->stream;
  // zeta and zeta**n_flow (n = 3) as in ufe_sia_solve, staged from the stack.
  double zc[2 * kMaxZ];
  for (int k = 0; k < nZ; ++k) { zc[k] = p->zeta[k]; zc[nZ + k] = std::pow(p->zeta[k], 3.0); }
  double *zeta = scratch, *zeta3 = scratch + nZ;
  // Ac intermediates the caller did not ask for go to the scratch. Every scratch word a
  // kernel reads is written earlier in the same call, so nothing needs clearing.
  double *edge = scratch + 2 * kMaxZ;
  const size_t na = nAc;
  double *D = out->D_SIA_Ac ? out->D_SIA_Ac : edge;
  double *Ux = out->Ux_SIA_Ac ? out->Ux_SIA_Ac : edge + na;
  double *Uy = out->Uy_SIA_Ac ? out->Uy_SIA_Ac : edge + 2 * na;
  double *Up = out->Up_SIA_Ac ? out->Up_SIA_Ac : edge + 3 * na;
  double *Uo = out->Uo_SIA_Ac ? out->Uo_SIA_Ac : edge + 4 * na;
  rc = cuda_status(cudaMemcpyAsync(zeta, zc, 2 * (size_t)nZ * sizeof(double), cudaMemcpyHostToDevice, s), "H2D zeta");
  if (!rc) {
    const unsigned g = (unsigned)((nAc + 255) / 256);
    if (nZ == 15)
      k_sia_edges<15><<<g, 256, 0, s>>>(nAc, nZ, in->mask_sheet_Ac, in->Hi_Ac, in->dHs_dx_Ac, in->dHs_dy_Ac,
                                        in->dHs_dp_Ac, in->dHs_do_Ac, in->A_flow_Ac, zeta, zeta3, p->m_enh_sia,
                                        out->D_SIA_3D_Ac, D, Ux, Uy, Up, Uo);
    else
      k_sia_edges<0><<<g, 256, 0, s>>>(nAc, nZ, in->mask_sheet_Ac, in->Hi_Ac, in->dHs_dx_Ac, in->dHs_dy_Ac,
                                       in->dHs_dp_Ac, in->dHs_do_Ac, in->A_flow_Ac, zeta, zeta3, p->m_enh_sia,
                                       out->D_SIA_3D_Ac, D, Ux, Uy, Up, Uo);
    rc = cuda_status(cudaGetLastError(), "k_sia_edges");
  }
  if (!rc && out->U_SIA) {
    k_ac_to_aa3<<<(unsigned)((nV + 255) / 256), 256, 0, s>>>(nV, m.nC, m.iAci, Ux, Uy, D, out->U_SIA, out->V_SIA,
                                                            out->D_SIA);
    rc = cuda_status(cudaGetLastError(), "k_ac_to_aa3");
  }
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "sia solve (no allocation)");
  return rc;
}
