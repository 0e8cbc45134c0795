// SSA velocity solve on the device: the whole Picard + coloured-SOR loop of solve_SSA in one
// persistent cooperative kernel, between one gather of the inputs and one scatter of the
// results. Convergence is decided on the device; no per-iteration host round trip.
//
// Reference routines (ice_dynamics_module.f90):
//   solve_SSA 408-557          Picard loop, RN test, reset handling          -> ssa_persistent
//   SSA_effective_viscosity 695-726 + get_mesh_derivatives_AaAc
//                              (mesh_ArakawaC_module.f90:583-618)            -> phase_viscosity
//   SSA_sliding_term 727-779 (+ linear law), centre coefficients and RHS 580-595
//                                                                            -> phase_coefficients
//   solve_SSA_linearised 597-691, five-colour SOR 607-664                    -> phase_sweep
//   apply_Neumann_boundary_AaAc (mesh_ArakawaC_module.f90:660-724)           -> phase_boundary
//   basal_yield_stress 780-844                                               -> k_gather
//   calculate_GL_flux 848-949                                                -> k_gl_flux
//   scatter 548-552 + rotate_xy_to_po (mesh_ArakawaC_module.f90:815-844)     -> k_scatter
//
// FP64 path: every multiply and add of the reference is evaluated in its order (the file is
// compiled with --fmad=false), with two precombined coefficient sets: (4Nxx+Nyy, 4Nyy+Nxx)
// per neighbour (the same doubles the reference forms each time) and the row sum of Nxy for
// the cross term, which the reference forms as U(ai)*Nxy(ai,1) + U(ai)*Nxy(ai,2) + ...
// (get_mesh_curvatures_vertex_AaAc multiplies the home value into every term).
//
// Mixed path: FP64 defect correction around FP32 sweeps. With u0 fixed (FP64), the defect
// r0 = b - A(eta) u0 is formed in FP64; the sweeps run the same coloured SOR on A d = r0 in
// FP32 from d = 0. SOR is affine-equivariant, so u0 + d follows the FP64 iterates exactly
// in exact arithmetic, and the residual the sweep tests against SSA_max_residual_UV is that
// of the FP64 iteration; FP32 rounding is relative to |d|, not |u|. Every `refold` sweeps
// d is folded into u0 and the defect recomputed in FP64. The viscosity uses FP32 arithmetic
// on FP64 differences u_j - u_i. Convergence norms (RN, max residual) are FP64. The mixed
// sweeps have no team barrier between sweeps: a sweep is decided one sweep later from a ring
// of per-sweep slots (lag_arrive / lag_decide), so a converged linear solve ends one sweep
// after the sweep that met the tolerance.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <utility>
#include <vector>

#include "ufe_internal.h"

namespace ufe {

// ---------------------------------------------------------------------------------------
// Control block and kernel arguments
// ---------------------------------------------------------------------------------------
struct SsaCtl {
  unsigned int bar_count;         // monotonic grid-barrier arrival counter (bit 30: error)
  int err;
  int status;
  int pad_;
  unsigned long long maxres[3];   // max |res| per sweep (ring of three), as ordered bits
  int picard_iterations;
  int linear_solves;
  int resets;
  int not_converged;
  long long total_sweeps;
  double last_RN;
  double last_max_residual;
  int sweeps[64];
  // lagged convergence decisions of the mixed sweeps (ring of kLagRing sweeps)
  unsigned long long lag_word[8];   // arrivals per slot, monotonic within a solve (lag_increment)
  unsigned long long lag_res[8];    // (sweep + 1) << 32 | FP32 bits of the sweep's max |res|, rounded up
};

// Sweep arithmetic of the persistent solver.
enum SweepMode : int {
  kExact64 = 0,   // the reference's expression order, no FMA, IEEE divisions
  kFast64 = 1,    // FP64 with fused multiply-adds and a per-Picard reciprocal of eu, ev
  kMixed = 2,     // FP32 correction sweeps inside FP64 defect correction
};

struct SsaArgs {
  // mesh
  const int *col;
  const double2 *cuv;
  const double2 *nxy;
  const float2 *cuv32;
  const float2 *nxy32;
  const uint8_t *deg;
  const int64_t *slice_ptr;
  const double2 *h_nxy;
  const double2 *h_cuv;
  const double *sNxy;
  const double *s3Nxy;
  const float2 *h_nxy32;
  const float *s3Nxy32;
  const int *bnd_ptr;
  const int *bnd_nbr;
  const int *slice_e0;
  const uint8_t *slice_w;
  const uint8_t *slice_g;
  const int *patch_slice;
  const int *patch_edge0;
  const int *edge_row;
  const int *sync_ptr;
  const int *sync_list;
  // halo sweep program (DevMesh, ufe_internal.h)
  const int *hp_slice, *hslice_e0;
  const int *hp_split;     // first slice of phase 0's rows that read halo slots
  const uint8_t *hslice_w;
  const int *hrow_l, *hrow_g;
  const uint16_t *hcol;
  const float2 *hcuv32;
  const double2 *hcuv;
  const int *hload_ptr, *hload_dev, *hsync_ptr, *hsync_list;
  const float *hs3_32;
  const double *hs3;
  float4 *hsd32;           // halo sweeps, mixed: per slot (1/eu, 1/ev, defect x, y) in FP32;
                           // boundary slots: (c0 x, c0 y, 1 / count, 0), see halo_boundary
  double2 *hrcp, *hrhs;    // halo sweeps, fast FP64: per slot (1/eu, 1/ev) and (RHSx, RHSy)
  float4 *bc0;             // mixed, per edge ordinal: (c0 x, c0 y, 1 / count, 0), see phase_boundary
  unsigned int *prog;      // per-CTA progress counters (stride 32 words)
  int n_edge;              // edge ordinals (edge rows and corners)
  int nP;
  int nSlices;
  int ncm;
  // fields in device row order
  const double *Hi, *Hb, *SL, *hx, *hy, *Af, *beta, *tau;
  const uint8_t *skip;    // Dirichlet rows (grounding-line Ac rows under the GL-flux option), may be null
  double2 *UV;            // FP64 velocities (u0 in the mixed path)
  float2 *dUV;            // mixed: correction d
  double2 *UVb, *UVc;     // halo sweeps, FP64 modes: the second and third velocity buffers
  float2 *dUVb, *dUVc;    // halo sweeps, mixed: the second and third correction buffers
  float2 *r0;             // mixed: defect
  float2 *rcp32;          // mixed: FP32 reciprocals of (eu, ev)
  double *eta, *Na, *Nb, *S;
  double2 *rhs, *euv, *rcp;
  double *rn_part;        // [2 * gridDim.x]
  SsaCtl *ctl;
  // parameters
  double omega, tol, rn_tol, m_enh, uq, expo, beta_const;
  int max_inner, max_outer, sliding_law, has_beta;
  int refold;
  int fp32_visc;
  int local_rows;          // keep the patch's own velocities (mixed: corrections) in shared memory
  int halo_index_off;      // halo sweeps: byte offset of the halo slots' device rows in dynamic shared memory
  int stage_off, stage_bytes;   // halo sweeps, mixed: the resident program slices' area in dynamic shared memory
  long long timeout_ns;
};

constexpr unsigned int kBarrierError = 1u << 30;
// Ring of the lagged decisions: a slot is reused kLagRing sweeps later, safe for lag <= 3
// (the writer of sweep G + kLagRing has seen every CTA finish sweep G + kLagRing - 1 - lag,
// after every reader of sweep G read it, when kLagRing > 2 lag + 1).
constexpr int kLagRing = 8;
constexpr int kMaxLag = 3;
// Mixed sweeps decide convergence this many sweeps late (0: a team barrier after every sweep).
#ifndef UFE_MIXED_LAG
#define UFE_MIXED_LAG 1
#endif
constexpr int kMixedLag = UFE_MIXED_LAG;
static_assert(kMixedLag >= 0 && kMixedLag <= kMaxLag, "lag out of range");
// Largest shared-memory mirror of a patch's rows (the rest of the 228 KB of an SM stays L1).
constexpr size_t kLocalRowsMaxBytes = 160 * 1024;
constexpr int kMaxKrylovRestart = 1000;   // largest GMRES restart length of the VJP
// Threads per CTA of the halo sweeps. Measured on the 200k dome: 1024 threads, one slice per
// warp at a time, 27.1 us per mixed sweep; 768 threads with two slices' loads issued together
// per warp (80 registers), 28.6 us.
#ifndef UFE_HALO_BLOCK
#define UFE_HALO_BLOCK 1024
#endif
constexpr int kHaloBlock = UFE_HALO_BLOCK;

// Per-phase timers of the persistent solver (profiling build only, -DUFE_PHASE_TIMERS=1):
// thread 0 of every CTA stamps clock64() at the end of each phase of the SOR loop (every
// phase ends with a CTA barrier, so its stamp is when the whole CTA is through) and adds the
// SM cycles since the previous stamp to a per-category total; the totals of all CTAs are
// summed into g_phase_cycles at the end of the launch. The normal build compiles none of it.
#ifndef UFE_PHASE_TIMERS
#define UFE_PHASE_TIMERS 0
#endif
enum PhaseTimer : int {
  kTmWaitColour = 0,   // neighbour waits before colour phases
  kTmColour,           // colour phases (sweep + publish)
  kTmArrive,           // the sweep's residual into the decision slot / block max
  kTmWaitBoundary,     // neighbour wait before the boundary phase
  kTmBoundary,         // boundary phase (+ publish)
  kTmDecide,           // reading lagged decisions
  kTmGrid,             // team barriers inside the SOR loop
  kTmOther,            // viscosity, RN, coefficients, defect, fold, refolds
  kTmSweeps,           // (count) sweeps of this CTA
  kTmColour0,          // halo sweeps: colour phases 1..5 one by one (also counted in kTmColour)
  kTmCount = kTmColour0 + 5
};
#if UFE_PHASE_TIMERS
__device__ unsigned long long g_phase_cycles[kTmCount];
constexpr int kTmMaxCta = 1024;
__device__ unsigned long long g_phase_cycles_cta[kTmMaxCta * kTmCount];   // per CTA, single solves
#define UFE_TM_DECL                                   \
  __shared__ unsigned long long s_tm[kTmCount];       \
  __shared__ long long s_tm0, s_tm1;                  \
  if (threadIdx.x < kTmCount) s_tm[threadIdx.x] = 0;  \
  if (threadIdx.x == 0) s_tm0 = s_tm1 = clock64();
#define UFE_TM(cat)                                               \
  do {                                                            \
    if (threadIdx.x == 0) {                                       \
      const long long now_ = clock64();                           \
      s_tm[cat] += (unsigned long long)(now_ - s_tm0);            \
      s_tm0 = s_tm1 = now_;                                       \
    }                                                             \
  } while (0)
// a sub-interval since the last stamp of either kind, without closing the current category
#define UFE_TM_SUB(cat)                                           \
  do {                                                            \
    if (threadIdx.x == 0) {                                       \
      const long long now_ = clock64();                           \
      s_tm[cat] += (unsigned long long)(now_ - s_tm1);            \
      s_tm1 = now_;                                               \
    }                                                             \
  } while (0)
#define UFE_TM_COUNT(cat) do { if (threadIdx.x == 0) s_tm[cat] += 1; } while (0)
#define UFE_TM_FLUSH()                                                                  \
  do {                                                                                  \
    __syncthreads();                                                                    \
    if (threadIdx.x < kTmCount) atomicAdd(&g_phase_cycles[threadIdx.x], s_tm[threadIdx.x]); \
    if (threadIdx.x < kTmCount && blockIdx.x < kTmMaxCta)                             \
      atomicAdd(&g_phase_cycles_cta[blockIdx.x * kTmCount + threadIdx.x], s_tm[threadIdx.x]); \
  } while (0)
#else
#define UFE_TM_DECL
#define UFE_TM(cat) do { } while (0)
#define UFE_TM_SUB(cat) do { } while (0)
#define UFE_TM_COUNT(cat) do { } while (0)
#define UFE_TM_FLUSH() do { } while (0)
#endif

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add_u32(unsigned int *p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// A team: the CTAs of a cooperative launch that solve one problem together. GridTeam is the
// whole grid (a single solve: rank and size come from the special registers, the counter
// from the constant-bank argument block, so the team costs no registers); SubTeam is a
// slice of the grid solving one ensemble member in the batched solver.
struct GridTeam {
  unsigned int *bar_;     // the monotonic barrier counter (bit 30: error)
  unsigned int epoch;     // barriers passed by this CTA
  __device__ __forceinline__ int rank() const { return (int)blockIdx.x; }
  __device__ __forceinline__ int size() const { return (int)gridDim.x; }
  __device__ __forceinline__ unsigned int *bar() const { return bar_; }
};
struct SubTeam {
  int rank_;              // this CTA's index in the team
  int size_;              // CTAs in the team
  unsigned int *bar_;
  unsigned int epoch;
  __device__ __forceinline__ int rank() const { return rank_; }
  __device__ __forceinline__ int size() const { return size_; }
  __device__ __forceinline__ unsigned int *bar() const { return bar_; }
};

// Team-wide barrier (every CTA of the team is co-resident): a monotonic arrival counter,
// epoch k is complete when the counter reaches k * size. The spin is bounded: after
// timeout_ns the CTA records UFE_TIMEOUT and sets the error bit in the counter, which
// releases every other waiter with a failure; callers then leave the kernel.
template <class Team>
__device__ __forceinline__ bool team_barrier(Team &t, int *err, long long timeout_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    t.epoch += 1u;   // only thread 0 arrives and waits
    const unsigned int target = t.epoch * (unsigned)t.size();
    // The CTA barrier above orders every thread's writes before thread 0's arrival, and the
    // release of the arrival is cumulative: it publishes them at GPU scope without a
    // separate fence.
    red_release_add_u32(t.bar(), 1u);
    unsigned int v = ld_acquire_u32(t.bar());
    if (!(v & kBarrierError) && (int)(v - target) < 0) {
      const unsigned long long t0 = globaltimer_ns();
      unsigned int ns = 16;
      for (;;) {
        __nanosleep(ns);
        if (ns < 128) ns <<= 1;
        v = ld_acquire_u32(t.bar());
        if ((v & kBarrierError) || (int)((v & ~kBarrierError) - target) >= 0) break;
        if ((long long)(globaltimer_ns() - t0) > timeout_ns) {
          atomicCAS(err, 0, (int)UFE_TIMEOUT);
          atomicOr(t.bar(), kBarrierError);
          v |= kBarrierError;
          break;
        }
      }
    }
    s_ok = (v & kBarrierError) == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block max of |res| bit patterns (the IEEE ordering of non-negative doubles equals the
// ordering of their bit patterns), then one atomicMax per CTA.
__device__ __forceinline__ void block_max_to(unsigned long long *dst, unsigned long long v) {
  __shared__ unsigned long long s_w[32];
  v = warp_max_u64(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) s_w[w] = v;
  __syncthreads();
  if (w == 0) {
    unsigned long long x = l < (int)(blockDim.x >> 5) ? s_w[l] : 0ull;
    x = warp_max_u64(x);
    if (l == 0 && x > 0ull) atomicMax(dst, x);
  }
  __syncthreads();
}

__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}

__device__ __forceinline__ bool is_floating(double Hi, double Hb, double SL) {
  return Hi < ((SL - Hb) * kSeawaterDensity) / kIceDensity;   // general_ice_model_data_module.f90:464-475
}

// ---------------------------------------------------------------------------------------
// Phases
// ---------------------------------------------------------------------------------------

// Effective viscosity and N = eta * max(0.1, H) on every row; block partial sums of
// (N - Nprev)^2 and N^2 for RN. FP64: reference order (home term first). FP32 variant
// (mixed path option): FP32 arithmetic on FP64 differences u_j - u_i.
template <class Team>
__device__ void phase_viscosity(const SsaArgs &a, const Team &t, double *N, const double *Nprev, bool fp32) {
  const int warps_per_block = blockDim.x >> 5;
  const int gw = t.rank() * warps_per_block + (threadIdx.x >> 5);
  const int nw = t.size() * warps_per_block;
  const int lane = threadIdx.x & 31;
  const int nslices = a.nP / kSlice;
  double sdn = 0.0, sn = 0.0;
  for (int s = gw; s < nslices; s += nw) {
    const int p = s * kSlice + lane;
    const int n = a.deg[p];
    if (n == 0) continue;
    const int64_t e0 = a.slice_ptr[s] + lane;
    const double2 ui = a.UV[p];
    double eta;
    if (!fp32) {
      const double2 h = a.h_nxy[p];
      double ux = h.x * ui.x, uy = h.y * ui.x, vx = h.x * ui.y, vy = h.y * ui.y;
      for (int k = 0; k < n; ++k) {
        const int64_t e = e0 + (int64_t)k * kSlice;
        const int j = a.col[e];
        const double2 c = a.nxy[e];
        const double2 uj = a.UV[j];
        ux = ux + c.x * uj.x;
        uy = uy + c.y * uj.x;
        vx = vx + c.x * uj.y;
        vy = vy + c.y * uj.y;
      }
      const double t = uy + vx;
      const double e2 = (((ux * ux + vy * vy) + ux * vy) + 0.25 * (t * t)) + 1e-12;
      eta = pow((a.m_enh * 0.5) * a.Af[p], -1.0 / 3.0) * pow(e2, (1.0 - 3.0) / (2.0 * 3.0));
    } else {
      // d/dx u = sum_k Nx_k (u_k - u_i) + u_i * (Nx_home + sum_k Nx_k); the row sum is zero
      // up to rounding (linear fields are reproduced exactly).
      const float2 rs = a.h_nxy32[p];
      float fux = rs.x * (float)ui.x, fuy = rs.y * (float)ui.x;
      float fvx = rs.x * (float)ui.y, fvy = rs.y * (float)ui.y;
      for (int k = 0; k < n; ++k) {
        const int64_t e = e0 + (int64_t)k * kSlice;
        const int j = a.col[e];
        const float2 c = a.nxy32[e];
        const double2 uj = a.UV[j];
        const float du = (float)(uj.x - ui.x), dv = (float)(uj.y - ui.y);
        fux = fmaf(c.x, du, fux);
        fuy = fmaf(c.y, du, fuy);
        fvx = fmaf(c.x, dv, fvx);
        fvy = fmaf(c.y, dv, fvy);
      }
      const float t = fuy + fvx;
      const float e2 = (((fux * fux + fvy * fvy) + fux * fvy) + 0.25f * (t * t)) + 1e-12f;
      eta = (double)(powf((float)((a.m_enh * 0.5) * a.Af[p]), -1.0f / 3.0f) * powf(e2, -1.0f / 3.0f));
    }
    const double Nn = eta * fmax(0.1, a.Hi[p]);
    a.eta[p] = eta;
    N[p] = Nn;
    const double dn = Nn - Nprev[p];
    sdn += dn * dn;
    sn += Nn * Nn;
  }
  // deterministic block reduction
  __shared__ double s_a[32], s_b[32];
  sdn = warp_sum(sdn);
  sn = warp_sum(sn);
  const int w = threadIdx.x >> 5;
  if (lane == 0) { s_a[w] = sdn; s_b[w] = sn; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0.0, y = 0.0;
    for (int k = 0; k < warps_per_block; ++k) { x += s_a[k]; y += s_b[k]; }
    a.rn_part[2 * t.rank()] = x;
    a.rn_part[2 * t.rank() + 1] = y;
  }
}

// RN = sqrt(sum (N - Nprev)^2 / sum N^2), reduced in a fixed order by every CTA.
template <class Team>
__device__ double final_rn(const SsaArgs &a, const Team &t) {
  __shared__ double s_rn;
  if (threadIdx.x < 32) {
    double x = 0.0, y = 0.0;
    for (int b = threadIdx.x; b < t.size(); b += 32) {
      x += *(volatile double *)&a.rn_part[2 * b];
      y += *(volatile double *)&a.rn_part[2 * b + 1];
    }
    x = warp_sum(x);
    y = warp_sum(y);
    if (threadIdx.x == 0) s_rn = sqrt(x / y);
  }
  __syncthreads();
  return s_rn;
}

// Sliding term S, centre coefficients (eu, ev), their reciprocals and the right-hand sides.
template <int kMode, class Team>
__device__ void phase_coefficients(const SsaArgs &a, const Team &t) {
  const int tid = t.rank() * blockDim.x + threadIdx.x;
  const int nt = t.size() * blockDim.x;
  for (int p = tid; p < a.nP; p += nt) {
    if (a.deg[p] == 0) continue;
    double S;
    if (a.sliding_law == UFE_SLIDING_COULOMB_REGULARISED) {
      const double2 u = a.UV[p];
      S = (a.tau[p] * pow((1e-3 * 1e-3 + u.x * u.x) + u.y * u.y, a.expo)) / a.uq;
    } else {
      S = a.has_beta ? a.beta[p] : a.beta_const;
    }
    a.S[p] = S;
    if (a.slice_g[p / kSlice] == 5) continue;   // edge rows are set by the boundary condition
    const double eta = a.eta[p];
    const double H = a.Hi[p];
    a.rhs[p] = make_double2(((kIceDensity * kGrav) * a.hx[p]) / eta, ((kIceDensity * kGrav) * a.hy[p]) / eta);
    const double2 h = a.h_cuv[p];
    double2 c;
    if (!is_floating(H, a.Hb[p], a.SL[p])) {
      c = make_double2(h.x - S / (fmax(0.1, H) * eta), h.y - S / (fmax(0.1, H) * eta));
    } else {
      c = h;
    }
    a.euv[p] = c;
    if (kMode != kExact64) {
      const double2 r = make_double2(1.0 / c.x, 1.0 / c.y);
      a.rcp[p] = r;
      if (kMode == kMixed) a.rcp32[p] = make_float2((float)r.x, (float)r.y);
    }
  }
}

// This CTA's patch: the first slice of each group, and per slice its first SELL entry and
// width, staged in shared memory at kernel start.
struct PatchSmem {
  int ps[kGroups + 1];
  int e0[kMaxPatchSlices];
  unsigned char w[kMaxPatchSlices];
  int edge0, edge1;
  int nsync;
  int sync[kMaxSync];
  // halo sweeps: program slices of the 7 phases (e0, w hold the program's slices), the own
  // device rows [p0, p0 + n_own) and the halo slots [n_own, n_own + nh) of the working copy
  int hps[8];
  int hsplit;   // phase 0: slices [hps[0], hsplit) read no halo slot
  int p0, n_own, nh, hl0;
  // lagged decisions: each slot's arrival word as this CTA last read it (lag_decide)
  unsigned long long lag_prev[8];
  int lag_act[2];
  unsigned long long lag_pre;   // the arrival word of sweep lag_pre_g, read ahead by lag_arrive_publish
  unsigned int lag_pre_g;
  // halo sweeps, mixed: offset (16-byte units) of each program slice's resident copy in the
  // staging area, -1 = read from global memory (halo_stage)
  short soff[kMaxPatchSlices];
};

// One colour of the FP64 sweep in the reference's expression order (parity mode).
__device__ unsigned long long phase_sweep_exact(const SsaArgs &a, const PatchSmem &ps, int g) {
  const int wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5, lane = threadIdx.x & 31;
  const double omega = a.omega;
  unsigned long long mx = 0ull;
  for (int s = ps.ps[g] + wid; s < ps.ps[g + 1]; s += nwarps) {
    const int p = s * kSlice + lane;
    const int n = a.deg[p];
    if (n == 0) continue;
    if (a.skip && a.skip[p]) continue;
    const int64_t e0 = ps.e0[s - ps.ps[0]] + lane;
    double su = 0.0, sv = 0.0;
    for (int k = 0; k < n; ++k) {
      const int64_t e = e0 + (int64_t)k * kSlice;
      const int j = a.col[e];
      const double2 c = a.cuv[e];
      const double2 u = a.UV[j];
      su = su + u.x * c.x;
      sv = sv + u.y * c.y;
    }
    const double2 ui = a.UV[p];
    const double sxy = a.sNxy[p];
    const double Uxy = ui.x * sxy, Vxy = ui.y * sxy;
    const double2 ec = a.euv[p];
    const double2 b = a.rhs[p];
    const double lhsx = (su + 3.0 * Vxy) + ec.x * ui.x;
    const double lhsy = (sv + 3.0 * Uxy) + ec.y * ui.y;
    const double ru = (lhsx - b.x) / ec.x;
    const double rv = (lhsy - b.y) / ec.y;
    const unsigned long long bu = abs_bits(ru), bv = abs_bits(rv);
    mx = bu > mx ? bu : mx;
    mx = bv > mx ? bv : mx;
    a.UV[p] = make_double2(ui.x - omega * ru, ui.y - omega * rv);
  }
  return mx;
}

constexpr int kBatch = 8;   // neighbour entries loaded in one batch (rows of higher degree load the rest)
// halo sweeps: warps that wait for the neighbouring patches and load the halo slots while the
// others run colour 1's halo-free rows (halo_fetch), and the loads each thread issues together
constexpr int kFetchWarps = 4;
constexpr int kFetchBatch = 4;

// One colour of the fast FP64 sweep: res = U + ((sum + 3 sNxy V) - RHS) / eu with the
// reciprocal of eu formed once per Picard iteration, products accumulated with FMA.
// Per row two dependent L2 round trips: (indices, coefficients, home values), then the
// neighbour gathers. Padding entries hold column -1.
// The patch's own rows [p0, p0 + n) mirrored in shared memory (n = 0: not mirrored). Rows
// of one patch are contiguous in device order and most neighbour reads of a sweep stay
// inside the patch, so they cost a shared-memory load instead of an L2 round trip; every
// write goes to both copies, so other patches and the grid-wide phases read global memory.
struct LocalRows {
  void *base;
  int p0;
  int n;
};

__device__ unsigned long long phase_sweep_fast(const SsaArgs &a, const PatchSmem &ps, int g, const LocalRows &lc) {
  const int wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5, lane = threadIdx.x & 31;
  const double omega = a.omega;
  unsigned long long mx = 0ull;
  for (int s = ps.ps[g] + wid; s < ps.ps[g + 1]; s += nwarps) {
    const int w = ps.w[s - ps.ps[0]];
    const int64_t e0 = ps.e0[s - ps.ps[0]] + lane;
    const int p = s * kSlice + lane;
    double2 *lu = static_cast<double2 *>(lc.base);
    int j[kBatch];
#pragma unroll
    for (int q = 0; q < kBatch; ++q) j[q] = q < w ? a.col[e0 + (int64_t)q * kSlice] : -1;
    const double2 ui = lc.n ? lu[p - lc.p0] : a.UV[p];
    const double s3 = a.s3Nxy[p];
    const double2 r = a.rcp[p];
    const double2 b = a.rhs[p];
    if (j[0] < 0 || (a.skip && a.skip[p])) continue;   // padding row, or a Dirichlet row
    double su = 0.0, sv = 0.0;
#pragma unroll
    for (int q = 0; q < kBatch; ++q) {
      if (j[q] >= 0) {
        const double2 c = a.cuv[e0 + (int64_t)q * kSlice];
        const unsigned o = (unsigned)(j[q] - lc.p0);
        const double2 u = o < (unsigned)lc.n ? lu[o] : a.UV[j[q]];
        su = fma(u.x, c.x, su);
        sv = fma(u.y, c.y, sv);
      }
    }
    for (int k = kBatch; k < w; ++k) {
      const int jj = a.col[e0 + (int64_t)k * kSlice];
      if (jj < 0) break;
      const double2 c = a.cuv[e0 + (int64_t)k * kSlice];
      const unsigned o = (unsigned)(jj - lc.p0);
      const double2 u = o < (unsigned)lc.n ? lu[o] : a.UV[jj];
      su = fma(u.x, c.x, su);
      sv = fma(u.y, c.y, sv);
    }
    const double ru = fma(fma(s3, ui.y, su) - b.x, r.x, ui.x);
    const double rv = fma(fma(s3, ui.x, sv) - b.y, r.y, ui.y);
    const unsigned long long bu = abs_bits(ru), bv = abs_bits(rv);
    mx = bu > mx ? bu : mx;
    mx = bv > mx ? bv : mx;
    const double2 un = make_double2(fma(-omega, ru, ui.x), fma(-omega, rv, ui.y));
    if (lc.n) lu[p - lc.p0] = un;
    a.UV[p] = un;
  }
  return mx;
}

// One colour of the FP32 correction sweep of the mixed path:
// res = d_i + ((sum_j c_j d_j + 3 sNxy d_i') - r0) / eu.
__device__ unsigned long long phase_sweep32(const SsaArgs &a, const PatchSmem &ps, int g, const LocalRows &lc) {
  const int wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5, lane = threadIdx.x & 31;
  const float omega = (float)a.omega;
  float mx = 0.0f;
  for (int s = ps.ps[g] + wid; s < ps.ps[g + 1]; s += nwarps) {
    const int w = ps.w[s - ps.ps[0]];
    const int64_t e0 = ps.e0[s - ps.ps[0]] + lane;
    const int p = s * kSlice + lane;
    int j[kBatch];
    float2 c[kBatch];
#pragma unroll
    for (int q = 0; q < kBatch; ++q) {
      j[q] = q < w ? a.col[e0 + (int64_t)q * kSlice] : -1;
      c[q] = q < w ? a.cuv32[e0 + (int64_t)q * kSlice] : make_float2(0.f, 0.f);
    }
    float2 *ld = static_cast<float2 *>(lc.base);
    const float2 di = lc.n ? ld[p - lc.p0] : a.dUV[p];
    const float s3 = a.s3Nxy32[p];
    const float2 r = a.rcp32[p];
    const float2 d = a.r0[p];
    if (j[0] < 0 || (a.skip && a.skip[p])) continue;   // padding row, or a Dirichlet row
    float2 u[kBatch];
#pragma unroll
    for (int q = 0; q < kBatch; ++q) {
      if (j[q] >= 0) {
        const unsigned o = (unsigned)(j[q] - lc.p0);
        u[q] = o < (unsigned)lc.n ? ld[o] : a.dUV[j[q]];
      }
    }
    float su = 0.0f, sv = 0.0f;
#pragma unroll
    for (int q = 0; q < kBatch; ++q) {
      if (j[q] >= 0) {
        su = fmaf(u[q].x, c[q].x, su);
        sv = fmaf(u[q].y, c[q].y, sv);
      }
    }
    for (int k = kBatch; k < w; ++k) {
      const int jj = a.col[e0 + (int64_t)k * kSlice];
      if (jj < 0) break;
      const float2 cc = a.cuv32[e0 + (int64_t)k * kSlice];
      const unsigned o = (unsigned)(jj - lc.p0);
      const float2 v = o < (unsigned)lc.n ? ld[o] : a.dUV[jj];
      su = fmaf(v.x, cc.x, su);
      sv = fmaf(v.y, cc.y, sv);
    }
    const float ru = fmaf(fmaf(s3, di.y, su) - d.x, r.x, di.x);
    const float rv = fmaf(fmaf(s3, di.x, sv) - d.y, r.y, di.y);
    mx = fmaxf(mx, fmaxf(fabsf(ru), fabsf(rv)));
    const float2 dn = make_float2(fmaf(-omega, ru, di.x), fmaf(-omega, rv, di.y));
    if (lc.n) ld[p - lc.p0] = dn;
    a.dUV[p] = dn;
  }
  return abs_bits((double)mx);
}

// Neumann boundary (apply_Neumann_boundary_AaAc): each edge row becomes the mean of its
// non-edge neighbours; the four corners the mean of all their neighbours, where an edge
// neighbour's new value is recomputed in place (same arithmetic, same result) so that the
// corners need no second pass. SUM(vals) in the reference runs over nC_mem slots whose
// unused entries are +0, hence the trailing "+ 0.0".
//
// Mixed path: with u = u0 + d on every row, the mean of the neighbours' u minus the row's u0
// is c0 + mean(d_j), c0 = mean(u0_j) - u0 (formed in FP64 by phase_defect whenever u0
// changes, stored per edge ordinal in bc0 as (c0 x, c0 y, 1 / count)), so a sweep's boundary
// phase is an FP32 sum of corrections and no FP64 division.
__device__ __forceinline__ double2 edge_mean(const SsaArgs &a, int k) {
  const int b0 = a.bnd_ptr[k], b1 = a.bnd_ptr[k + 1];
  double sx = 0.0, sy = 0.0;
  for (int q = b0; q < b1; ++q) {
    const double2 u = a.UV[a.bnd_nbr[q]];
    sx = sx + u.x;
    sy = sy + u.y;
  }
  const int nvals = b1 - b0;
  if (nvals < a.ncm) { sx = sx + 0.0; sy = sy + 0.0; }
  return make_double2(sx / (double)nvals, sy / (double)nvals);
}

__device__ __forceinline__ float2 edge_correction(const SsaArgs &a, int k) {
  const int b0 = a.bnd_ptr[k], b1 = a.bnd_ptr[k + 1];
  const float4 c = a.bc0[k];
  float sx = 0.0f, sy = 0.0f;
  for (int q = b0; q < b1; ++q) {
    const float2 d = a.dUV[a.bnd_nbr[q]];
    sx = sx + d.x;
    sy = sy + d.y;
  }
  return make_float2(fmaf(sx, c.z, c.x), fmaf(sy, c.z, c.y));
}

template <bool kM>
__device__ void phase_boundary(const SsaArgs &a, const PatchSmem &ps, const LocalRows &lc) {
  for (int k = ps.edge0 + threadIdx.x; k < ps.edge1; k += blockDim.x) {
    const int p = a.edge_row[k];
    const int b0 = a.bnd_ptr[k], b1 = a.bnd_ptr[k + 1];
    if constexpr (kM) {
      const float4 c = a.bc0[k];
      float sx = 0.0f, sy = 0.0f;
      for (int q = b0; q < b1; ++q) {
        const int j = a.bnd_nbr[q];
        // a corner's edge neighbour: its new correction, recomputed
        const float2 d = j < 0 ? edge_correction(a, -j - 1) : a.dUV[j];
        sx = sx + d.x;
        sy = sy + d.y;
      }
      const float2 dv = make_float2(fmaf(sx, c.z, c.x), fmaf(sy, c.z, c.y));
      a.dUV[p] = dv;
      if (lc.n) static_cast<float2 *>(lc.base)[p - lc.p0] = dv;
    } else {
      double sx = 0.0, sy = 0.0;
      for (int q = b0; q < b1; ++q) {
        const int j = a.bnd_nbr[q];
        const double2 u = j < 0 ? edge_mean(a, -j - 1) : a.UV[j];   // a corner's edge neighbour, recomputed
        sx = sx + u.x;
        sy = sy + u.y;
      }
      const int nvals = b1 - b0;
      if (nvals < a.ncm) { sx = sx + 0.0; sy = sy + 0.0; }
      const double2 v = make_double2(sx / (double)nvals, sy / (double)nvals);
      a.UV[p] = v;
      if (lc.n) static_cast<double2 *>(lc.base)[p - lc.p0] = v;
    }
  }
}

// ---------------------------------------------------------------------------------------
// Halo sweeps: one phase of the sweep program over this patch's working copy `ld` (shared
// memory; own rows, then halo rows). Every update uses the arithmetic, and the neighbour
// order, of the phased sweeps above, so an own row gets the same value either way; own rows
// are also written to `out` (the buffer the neighbours read at the next sweep's start) and
// alone enter the maximum residual.
// ---------------------------------------------------------------------------------------
constexpr uint16_t kNoCol = 0xffff;

__device__ __forceinline__ int halo_global(const SsaArgs &a, const PatchSmem &ps, int l) {
  return l < ps.n_own ? ps.p0 + l : a.hload_dev[ps.hl0 + l - ps.n_own];
}

// One slice of a colour phase of the FP32 correction sweep (as phase_sweep32), its entries
// read through pointers already offset by the lane (entry k of the lane at [32 k]).
__device__ __forceinline__ void slice32(const SsaArgs &a, const PatchSmem &ps, int w, const uint16_t *pc,
                                        const float2 *pcu, int l, float s3, float4 sd, const int *hidx, float2 *ld,
                                        float2 *out, float omega, float &mx) {
  int j[kBatch];
  float2 c[kBatch];
#pragma unroll
  for (int q = 0; q < kBatch; ++q) {
    j[q] = q < w ? (int)pc[q * kSlice] : (int)kNoCol;
    c[q] = q < w ? pcu[q * kSlice] : make_float2(0.f, 0.f);
  }
  if (l < 0) return;   // padding slot
  if (a.skip && a.skip[l < ps.n_own ? ps.p0 + l : hidx[l - ps.n_own]]) return;   // a Dirichlet row
  const float2 di = ld[l];
  float su = 0.0f, sv = 0.0f;
#pragma unroll
  for (int q = 0; q < kBatch; ++q) {
    if (j[q] != (int)kNoCol) {
      const float2 u = ld[j[q]];
      su = fmaf(u.x, c[q].x, su);
      sv = fmaf(u.y, c[q].y, sv);
    }
  }
  for (int k = kBatch; k < w; ++k) {
    const int jj = pc[k * kSlice];
    if (jj == (int)kNoCol) break;
    const float2 cc = pcu[k * kSlice];
    const float2 v = ld[jj];
    su = fmaf(v.x, cc.x, su);
    sv = fmaf(v.y, cc.y, sv);
  }
  const float ru = fmaf(fmaf(s3, di.y, su) - sd.z, sd.x, di.x);
  const float rv = fmaf(fmaf(s3, di.x, sv) - sd.w, sd.y, di.y);
  const float2 dn = make_float2(fmaf(-omega, ru, di.x), fmaf(-omega, rv, di.y));
  ld[l] = dn;
  if (l < ps.n_own) {
    out[ps.p0 + l] = dn;
    mx = fmaxf(mx, fmaxf(fabsf(ru), fabsf(rv)));
  }
}

// Colour phase f of the FP32 correction sweep: warp w takes slices w, w + nwarps, ... (a
// colour of a 200k-vertex patch has 42-50 slices for 32 warps). A round of 32 slices costs
// about 0.5 us plus the time to bring its program data (about 100 KB) from L2 into the SM,
// which is why the resident slices (halo_stage) are read from shared memory.
__device__ unsigned long long halo_colour32(const SsaArgs &a, const PatchSmem &ps, int s_begin, int s_end, int nwarps,
                                            const unsigned char *stage, const int *hidx, float2 *ld, float2 *out) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float omega = (float)a.omega;
  float mx = 0.0f;
  const int base = ps.hps[0];
  for (int s = s_begin + wid; s < s_end; s += nwarps) {
    const int w = ps.w[s - base];
    const int so = ps.soff[s - base];
    if (so >= 0) {
      const unsigned char *b = stage + 16 * so;
      const int *rl = reinterpret_cast<const int *>(b + w * kSlice * 10);
      slice32(a, ps, w, reinterpret_cast<const uint16_t *>(b) + lane, reinterpret_cast<const float2 *>(b + w * kSlice * 2) + lane,
              rl[lane], reinterpret_cast<const float *>(rl)[kSlice + lane], reinterpret_cast<const float4 *>(rl + 2 * kSlice)[lane],
              hidx, ld, out, omega, mx);
    } else {
      const int64_t e0 = ps.e0[s - base] + lane;
      const int slot = s * kSlice + lane;
      slice32(a, ps, w, a.hcol + e0, a.hcuv32 + e0, a.hrow_l[slot], a.hs3_32[slot], a.hsd32[slot], hidx, ld, out, omega,
              mx);
    }
  }
  return abs_bits((double)mx);
}

// Resident program slices (mixed halo sweeps). The shared memory left after the working copy
// and the halo indices (stage_bytes) holds, for the whole solve, copies of some of the patch's
// colour-phase slices: the entries' local columns and coefficients, then per slot the local row,
// 3 sNxy and the row data of halo_refresh (refreshed there with the global copy): w * 320 + 768
// bytes for a slice of width w. Which: whole rounds (a slice per warp: 32 slices, 28 for colour
// 1's halo-free rows, which four warps leave to the halo fetch), smallest first — the rounds after
// the first of a colour, and whole colours of at most one round (colour 1 counting as two: its
// halo-free rows and the others) — as many as fit. Thread 0 plans, then the CTA copies the static
// parts.
__device__ __forceinline__ int stage_slice_bytes(int w) { return w * kSlice * 10 + 2 * kSlice * 4 + kSlice * 16; }

__device__ void halo_stage(const SsaArgs &a, PatchSmem &ps, unsigned char *stage) {
  const int base = ps.hps[0];
  for (int s = ps.hps[0] + (int)threadIdx.x; s < ps.hps[7]; s += blockDim.x) ps.soff[s - base] = -1;
  __syncthreads();
  constexpr int kMaxUnits = 40;
  __shared__ int u0[kMaxUnits], u1[kMaxUnits], ub[kMaxUnits];
  if (threadIdx.x == 0 && a.stage_bytes > 0) {
    int nu = 0;
    for (int f = -1; f < 5; ++f) {   // -1: colour 1's halo-free rows, 0: its other rows
      const int s0 = f < 0 ? ps.hps[0] : f == 0 ? ps.hsplit : ps.hps[f];
      const int s1 = f < 0 ? ps.hsplit : ps.hps[f + 1];
      const int rs = (int)(blockDim.x >> 5) - (f < 0 ? kFetchWarps : 0);   // slices per round
      for (int r = s1 - s0 <= rs ? s0 : s0 + rs; r < s1 && nu < kMaxUnits; r += rs) {
        u0[nu] = r;
        u1[nu] = r + rs < s1 ? r + rs : s1;
        int b = 0;
        for (int q = u0[nu]; q < u1[nu]; ++q) b += stage_slice_bytes(ps.w[q - base]);
        ub[nu++] = b;
      }
    }
    int used = 0;
    for (;;) {
      int best = -1;
      for (int k = 0; k < nu; ++k)
        if (ub[k] >= 0 && (best < 0 || ub[k] < ub[best])) best = k;
      if (best < 0 || used + ub[best] > a.stage_bytes) break;
      for (int q = u0[best]; q < u1[best]; ++q) {
        ps.soff[q - base] = (short)(used / 16);
        used += stage_slice_bytes(ps.w[q - base]);
      }
      ub[best] = -1;
    }
  }
  __syncthreads();
  const int wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (int s = ps.hps[0] + wid; s < ps.hps[5]; s += nwarps) {
    const int so = ps.soff[s - base];
    if (so < 0) continue;
    unsigned char *b = stage + 16 * so;
    const int w = ps.w[s - base];
    const int64_t e0 = ps.e0[s - base];
    uint16_t *pc = reinterpret_cast<uint16_t *>(b);
    float2 *pcu = reinterpret_cast<float2 *>(b + w * kSlice * 2);
    for (int k = lane; k < w * kSlice; k += kSlice) {
      pc[k] = a.hcol[e0 + k];
      pcu[k] = a.hcuv32[e0 + k];
    }
    int *rl = reinterpret_cast<int *>(b + w * kSlice * 10);
    rl[lane] = a.hrow_l[s * kSlice + lane];
    reinterpret_cast<float *>(rl)[kSlice + lane] = a.hs3_32[s * kSlice + lane];
  }
  __syncthreads();
}

// Colour phase f of the FP64 sweeps (as phase_sweep_exact and phase_sweep_fast).
template <bool kExact>
__device__ unsigned long long halo_colour64(const SsaArgs &a, const PatchSmem &ps, int s_begin, int s_end, int nwarps,
                                            double2 *ld, double2 *out) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double omega = a.omega;
  unsigned long long mx = 0ull;
  const int base = ps.hps[0];
  for (int s = s_begin + wid; s < s_end; s += nwarps) {
    const int w = ps.w[s - base];
    const int64_t e0 = ps.e0[s - base] + lane;
    const int slot = s * kSlice + lane;
    const int l = a.hrow_l[slot];
    const int g = a.hrow_g[slot];
    if (l < 0 || (a.skip && a.skip[g])) continue;
    double su = 0.0, sv = 0.0;
    double ru, rv;
    const double2 ui = ld[l];
    if (kExact) {
      for (int k = 0; k < w; ++k) {
        const int64_t e = e0 + (int64_t)k * kSlice;
        const int jj = a.hcol[e];
        if (jj == (int)kNoCol) break;
        const double2 c = a.hcuv[e];
        const double2 u = ld[jj];
        su = su + u.x * c.x;
        sv = sv + u.y * c.y;
      }
      const double sxy = a.sNxy[g];
      const double Uxy = ui.x * sxy, Vxy = ui.y * sxy;
      const double2 ec = a.euv[g];
      const double2 b = a.rhs[g];
      const double lhsx = (su + 3.0 * Vxy) + ec.x * ui.x;
      const double lhsy = (sv + 3.0 * Uxy) + ec.y * ui.y;
      ru = (lhsx - b.x) / ec.x;
      rv = (lhsy - b.y) / ec.y;
    } else {
      int j[kBatch];
#pragma unroll
      for (int q = 0; q < kBatch; ++q) j[q] = q < w ? (int)a.hcol[e0 + (int64_t)q * kSlice] : (int)kNoCol;
      const double s3 = a.hs3[slot];
      const double2 r = a.hrcp[slot];
      const double2 b = a.hrhs[slot];
#pragma unroll
      for (int q = 0; q < kBatch; ++q) {
        if (j[q] != (int)kNoCol) {
          const double2 c = a.hcuv[e0 + (int64_t)q * kSlice];
          const double2 u = ld[j[q]];
          su = fma(u.x, c.x, su);
          sv = fma(u.y, c.y, sv);
        }
      }
      for (int k = kBatch; k < w; ++k) {
        const int jj = a.hcol[e0 + (int64_t)k * kSlice];
        if (jj == (int)kNoCol) break;
        const double2 c = a.hcuv[e0 + (int64_t)k * kSlice];
        const double2 u = ld[jj];
        su = fma(u.x, c.x, su);
        sv = fma(u.y, c.y, sv);
      }
      ru = fma(fma(s3, ui.y, su) - b.x, r.x, ui.x);
      rv = fma(fma(s3, ui.x, sv) - b.y, r.y, ui.y);
    }
    const double2 un = kExact ? make_double2(ui.x - omega * ru, ui.y - omega * rv)
                              : make_double2(fma(-omega, ru, ui.x), fma(-omega, rv, ui.y));
    ld[l] = un;
    if (l < ps.n_own) {
      out[g] = un;
      const unsigned long long bu = abs_bits(ru), bv = abs_bits(rv);
      mx = bu > mx ? bu : mx;
      mx = bv > mx ? bv : mx;
    }
  }
  return mx;
}

// Boundary phase f (5: edge rows, 6: corners) of apply_Neumann_boundary_AaAc: the mean of the
// listed neighbours (edge rows: the non-edge ones; corners: all, the edge rows among them
// already updated in phase 5), as phase_boundary. Every load of a slot is issued before any is
// used (an edge row averages at most a few neighbours), so a phase costs one round trip.
// Mixed: with u0 fixed between refolds, mean(u0_j + d_j) - u0_i = c0_i + mean(d_j), where
// c0_i = mean(u0_j) - u0_i is formed in FP64 at the refresh; the sweep then adds the FP32
// corrections only.
template <bool kM, class T>
__device__ void halo_boundary(const SsaArgs &a, const PatchSmem &ps, int f, T *ld, T *out) {
  const int wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5, lane = threadIdx.x & 31;
  const int base = ps.hps[0];
  constexpr int kB = 4;
  for (int s = ps.hps[f] + wid; s < ps.hps[f + 1]; s += nwarps) {
    const int w = ps.w[s - base];
    const int64_t e0 = ps.e0[s - base] + lane;
    const int slot = s * kSlice + lane;
    const int l = a.hrow_l[slot];
    const int g = a.hrow_g[slot];
    int jb[kB];
#pragma unroll
    for (int k = 0; k < kB; ++k) jb[k] = k < w ? (int)a.hcol[e0 + (int64_t)k * kSlice] : (int)kNoCol;
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (kM) c = a.hsd32[slot];
    if (l < 0) continue;
    T nv;
    if constexpr (kM) {
      float sx = 0.0f, sy = 0.0f;
#pragma unroll
      for (int k = 0; k < kB; ++k)
        if (jb[k] != (int)kNoCol) {
          const float2 dj = ld[jb[k]];
          sx = sx + dj.x;
          sy = sy + dj.y;
        }
      for (int k = kB; k < w; ++k) {
        const int jj = a.hcol[e0 + (int64_t)k * kSlice];
        if (jj == (int)kNoCol) break;
        const float2 dj = ld[jj];
        sx = sx + dj.x;
        sy = sy + dj.y;
      }
      nv = make_float2(fmaf(sx, c.z, c.x), fmaf(sy, c.z, c.y));
    } else {
      // the packed entries in the reference's order (padding only after the last)
      double sx = 0.0, sy = 0.0;
      int nvals = 0;
#pragma unroll
      for (int k = 0; k < kB; ++k)
        if (jb[k] != (int)kNoCol) {
          const double2 u = ld[jb[k]];
          sx = sx + u.x;
          sy = sy + u.y;
          ++nvals;
        }
      for (int k = kB; k < w; ++k) {
        const int jj = a.hcol[e0 + (int64_t)k * kSlice];
        if (jj == (int)kNoCol) break;
        const double2 u = ld[jj];
        sx = sx + u.x;
        sy = sy + u.y;
        ++nvals;
      }
      if (nvals < a.ncm) { sx = sx + 0.0; sy = sy + 0.0; }
      nv = make_double2(sx / (double)nvals, sy / (double)nvals);
    }
    ld[l] = nv;
    if (l < ps.n_own) out[g] = nv;
  }
}

// Per-slot copies of the row data a sweep reads that change between linear solves (mixed:
// the FP32 reciprocals of the centre coefficients and the defect; fast FP64: the reciprocals
// and the right-hand side), refreshed by each CTA for its own program slots once the
// grid-wide phase that wrote them is complete.
template <int kMode>
__device__ __forceinline__ void halo_refresh(const SsaArgs &a, const PatchSmem &ps, unsigned char *stage) {
  for (int k = 32 * ps.hps[0] + (int)threadIdx.x; k < 32 * ps.hps[7]; k += blockDim.x) {
    if (a.hrow_l[k] < 0) continue;
    const int g = a.hrow_g[k];
    if constexpr (kMode == kMixed) {
      const float2 r = a.rcp32[g], d = a.r0[g];
      a.hsd32[k] = make_float4(r.x, r.y, d.x, d.y);
      if (k < 32 * ps.hps[5]) {
        const int s = k / kSlice, so = ps.soff[s - ps.hps[0]];
        if (so >= 0)
          reinterpret_cast<float4 *>(stage + 16 * so + ps.w[s - ps.hps[0]] * kSlice * 10 + 2 * kSlice * 4)[k % kSlice] =
              make_float4(r.x, r.y, d.x, d.y);
      }
      if (k >= 32 * ps.hps[5]) {
        // boundary slots: c0 = mean of the averaged neighbours' u0 minus the row's u0 (FP64),
        // and 1 / (number averaged), for halo_boundary
        const int s = k / kSlice, lane = k % kSlice;
        const int w = ps.w[s - ps.hps[0]];
        const int64_t e0 = ps.e0[s - ps.hps[0]] + lane;
        double sx = 0.0, sy = 0.0;
        int n = 0;
        for (int q = 0; q < w; ++q) {
          const int jj = a.hcol[e0 + (int64_t)q * kSlice];
          if (jj == (int)kNoCol) break;
          const double2 u = a.UV[halo_global(a, ps, jj)];
          sx = sx + u.x;
          sy = sy + u.y;
          ++n;
        }
        const double2 u0 = a.UV[g];
        const double rn = n > 0 ? 1.0 / (double)n : 0.0;
        a.hsd32[k] = make_float4((float)(sx * rn - u0.x), (float)(sy * rn - u0.y), (float)rn, 0.0f);
      }
    } else {
      a.hrcp[k] = a.rcp[g];
      a.hrhs[k] = a.rhs[g];
    }
  }
  __syncthreads();
}

// Halo slots of the working copy from the buffer the neighbours wrote in the last sweep.
// The patch's halo slots' device rows are kept in shared memory after the working copy
// (halo_index), which saves one dependent L2 load per sweep.
template <class T>
__device__ __forceinline__ void halo_load(const PatchSmem &ps, const int *hidx, T *ld, const T *in) {
  for (int i = threadIdx.x; i < ps.nh; i += blockDim.x) ld[ps.n_own + i] = in[hidx[i]];
}

// Own rows of the working copy into a global buffer.
template <class T>
__device__ __forceinline__ void halo_store_own(const PatchSmem &ps, const T *ld, T *dst) {
  for (int i = threadIdx.x; i < ps.n_own; i += blockDim.x) dst[ps.p0 + i] = ld[i];
}

// Mixed path: u0 += d, d = 0 on every row.
template <class Team>
__device__ void phase_fold(const SsaArgs &a, const Team &t) {
  const int tid = t.rank() * blockDim.x + threadIdx.x;
  const int nt = t.size() * blockDim.x;
  for (int p = tid; p < a.nP; p += nt) {
    const float2 d = a.dUV[p];
    if (d.x != 0.0f || d.y != 0.0f) {
      double2 u = a.UV[p];
      u.x = u.x + (double)d.x;
      u.y = u.y + (double)d.y;
      a.UV[p] = u;
      a.dUV[p] = make_float2(0.0f, 0.0f);
    }
  }
}

// Mixed path: FP64 defect r0 = RHS - LHS(u0) on the swept rows (streamed coefficient loads).
template <class Team>
__device__ void phase_defect(const SsaArgs &a, const Team &t) {
  const int warps_per_block = blockDim.x >> 5;
  const int gw = t.rank() * warps_per_block + (threadIdx.x >> 5);
  const int nw = t.size() * warps_per_block;
  const int lane = threadIdx.x & 31;
  for (int s = gw; s < a.nSlices; s += nw) {
    if (a.slice_g[s] == 5) continue;
    const int p = s * kSlice + lane;
    const int n = a.deg[p];
    if (n == 0) continue;
    const int64_t e0 = a.slice_ptr[s] + lane;
    double su = 0.0, sv = 0.0;
    for (int k = 0; k < n; ++k) {
      const int64_t e = e0 + (int64_t)k * kSlice;
      const int j = __ldcs(a.col + e);
      const double2 c = __ldcs(a.cuv + e);
      const double2 u = a.UV[j];
      su = fma(u.x, c.x, su);
      sv = fma(u.y, c.y, sv);
    }
    const double2 ui = a.UV[p];
    const double s3 = a.s3Nxy[p];
    const double2 ec = a.euv[p];
    const double2 b = a.rhs[p];
    const double lhsx = fma(ec.x, ui.x, fma(s3, ui.y, su));
    const double lhsy = fma(ec.y, ui.y, fma(s3, ui.x, sv));
    a.r0[p] = make_float2((float)(b.x - lhsx), (float)(b.y - lhsy));
  }
  // the boundary offsets of the new u0 (phase_boundary): c0 = mean of the averaged
  // neighbours' u0 minus the row's u0, in FP64; a corner's edge neighbour by its row
  const int tid = t.rank() * blockDim.x + threadIdx.x;
  const int nt = t.size() * blockDim.x;
  for (int k = tid; k < a.n_edge; k += nt) {
    const int b0 = a.bnd_ptr[k], b1 = a.bnd_ptr[k + 1];
    double sx = 0.0, sy = 0.0;
    for (int q = b0; q < b1; ++q) {
      const int j = a.bnd_nbr[q];
      const double2 u = a.UV[j < 0 ? a.edge_row[-j - 1] : j];
      sx = sx + u.x;
      sy = sy + u.y;
    }
    const double2 u0 = a.UV[a.edge_row[k]];
    const int n = b1 - b0;
    const double rn = n > 0 ? 1.0 / (double)n : 0.0;
    a.bc0[k] = make_float4((float)(sx * rn - u0.x), (float)(sy * rn - u0.y), (float)rn, 0.0f);
  }
}

template <class Team>
__device__ void phase_zero_velocity(const SsaArgs &a, const Team &t, bool mixed) {
  const int tid = t.rank() * blockDim.x + threadIdx.x;
  const int nt = t.size() * blockDim.x;
  for (int p = tid; p < a.nP; p += nt) {
    a.UV[p] = make_double2(0.0, 0.0);
    if (mixed) a.dUV[p] = make_float2(0.0f, 0.0f);
  }
}

// ---------------------------------------------------------------------------------------
// The persistent solver
// ---------------------------------------------------------------------------------------

// Progress of this CTA's patch: the number of colour phases it has completed in this launch.
template <class Args, class Team>
__device__ __forceinline__ void publish_progress(const Args &a, const Team &t, unsigned int value) {
  __syncthreads();
  if (threadIdx.x == 0) {   // cumulative release after the CTA barrier (see team_barrier)
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a.prog + 32 * t.rank()), "r"(value) : "memory");
  }
}

// Wait until every patch this patch synchronises with has completed `target` colour phases.
// Bounded: after timeout_ns the CTA records UFE_TIMEOUT and sets the team's error bit, which
// ends every other wait of the team (and the next team barrier or lagged decision fails).
template <class Args>
__device__ __forceinline__ void wait_neighbours(const Args &a, const PatchSmem &ps, unsigned int target,
                                                unsigned int *team_bar) {
  if (threadIdx.x < ps.nsync) {
    const unsigned int *q = a.prog + 32 * ps.sync[threadIdx.x];
    unsigned int v = ld_acquire_u32(q);
    if ((int)(v - target) < 0) {
      const unsigned long long t0 = globaltimer_ns();
      unsigned int ns = 16;
      for (;;) {
        __nanosleep(ns);
        if (ns < 64) ns <<= 1;
        v = ld_acquire_u32(q);
        if ((int)(v - target) >= 0) break;
        if (*(volatile unsigned int *)team_bar & kBarrierError) break;   // another CTA failed
        if ((long long)(globaltimer_ns() - t0) > a.timeout_ns) {
          atomicCAS(&a.ctl->err, 0, (int)UFE_TIMEOUT);
          atomicOr(team_bar, kBarrierError);
          break;
        }
      }
    }
  }
  __syncthreads();
}

// wait_neighbours and halo_load by the last kFetchWarps warps (the others meanwhile run the
// rows that read no halo slot); the caller's CTA barrier then orders the halo slots before their
// readers. The loads of a thread are issued together (up to kFetchBatch in flight).
template <class T>
__device__ __forceinline__ void halo_fetch(const SsaArgs &a, const PatchSmem &ps, unsigned int target,
                                           unsigned int *team_bar, bool wait, const int *hidx, T *ld, const T *in) {
  const int ft = (int)threadIdx.x - (int)(blockDim.x - kFetchWarps * kSlice);   // 0 .. 127
  if (wait) {
    for (int i = ft; i < ps.nsync; i += kFetchWarps * kSlice) {
      const unsigned int *q = a.prog + 32 * ps.sync[i];
      unsigned int v = ld_acquire_u32(q);
      if ((int)(v - target) < 0) {
        const unsigned long long t0 = globaltimer_ns();
        unsigned int ns = 16;
        for (;;) {
          __nanosleep(ns);
          if (ns < 64) ns <<= 1;
          v = ld_acquire_u32(q);
          if ((int)(v - target) >= 0) break;
          if (*(volatile unsigned int *)team_bar & kBarrierError) break;   // another CTA failed
          if ((long long)(globaltimer_ns() - t0) > a.timeout_ns) {
            atomicCAS(&a.ctl->err, 0, (int)UFE_TIMEOUT);
            atomicOr(team_bar, kBarrierError);
            break;
          }
        }
      }
    }
    // the fetch warps' barrier (id 1) orders every acquire before their halo loads
    asm volatile("bar.sync 1, %0;" ::"r"(kFetchWarps * kSlice) : "memory");
  }
  constexpr int kStride = kFetchWarps * kSlice;
  for (int i0 = ft; i0 < ps.nh; i0 += kStride * kFetchBatch) {
    T v[kFetchBatch];
#pragma unroll
    for (int k = 0; k < kFetchBatch; ++k) {
      const int i = i0 + k * kStride;
      if (i < ps.nh) v[k] = in[hidx[i]];
    }
#pragma unroll
    for (int k = 0; k < kFetchBatch; ++k) {
      const int i = i0 + k * kStride;
      if (i < ps.nh) ld[ps.n_own + i] = v[k];
    }
  }
}

// Lagged decisions (mixed sweeps). After its colour phases each CTA folds its maximum |res|
// into the ring slot of sweep G (one atomicMax of a key that carries the sweep, kept for the
// report of the final residual) and, behind a release, adds its arrival to the slot's word:
// 1 (the count, bits 0-15), plus 1 << 16 unless its residual is below the tolerance, 1 << 32 if
// it is above 1e6 (divergence), 1 << 48 if it is NaN. The residual travels as FP32 rounded up,
// so a decision can only come later, never earlier, than the FP64 value would give. A reader
// takes the difference between the word and the value it read at the slot's previous use: once
// the count there is the team's size, the three counts decide the sweep as the maximum would
// (converged when none is at or above the tolerance; diverged when some are above 1e6; neither
// when some are NaN) with a single load. Every CTA reads every sweep of a solve in order (the
// sweeps left undecided at the end of a linear solve are drained), so that difference holds
// exactly the sweep's arrivals; a count above the team's size means that the slot was refilled
// before it was read (cannot happen with lag <= kMaxLag). The halo sweeps' arrival reads the
// previous sweep's word ahead, its load overlapping the arrival's fence, and the decision uses
// that value when it already holds the whole sweep.
__device__ __forceinline__ unsigned long long lag_increment(unsigned long long mx_bits, double tol, unsigned int G,
                                                            unsigned long long *key) {
  const float r = __double2float_ru(__longlong_as_double((long long)mx_bits));
  *key = ((unsigned long long)(G + 1u) << 32) | (unsigned long long)__float_as_uint(r);
  const double rd = (double)r;
  unsigned long long inc = 1ull;
  if (!(rd < tol)) inc += 1ull << 16;
  if (rd > 1e6) inc += 1ull << 32;
  if (rd != rd) inc += 1ull << 48;
  return inc;
}

__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v) {
  __shared__ unsigned long long s_w[32];
  v = warp_max_u64(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) s_w[w] = v;
  __syncthreads();
  unsigned long long x = 0ull;
  if (w == 0) {
    x = l < (int)(blockDim.x >> 5) ? s_w[l] : 0ull;
    x = warp_max_u64(x);
  }
  return x;   // valid in thread 0
}

__device__ __forceinline__ void lag_arrive(const SsaArgs &a, unsigned int G, unsigned long long mx_bits) {
  const unsigned long long x = block_max_u64(mx_bits);
  if (threadIdx.x == 0) {
    unsigned long long key;
    const unsigned long long inc = lag_increment(x, a.tol, G, &key);
    atomicMax(&a.ctl->lag_res[G % kLagRing], key);
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(&a.ctl->lag_word[G % kLagRing]), "l"(inc) : "memory");
  }
}

// lag_arrive, then publish_progress(value), under one release: a single fence orders the
// slot's maximum, and every write of the CTA before the barrier, before both the arrival and
// the progress counter (a fence followed by relaxed writes is a release of each of them).
template <class Team>
__device__ __forceinline__ void lag_arrive_publish(const SsaArgs &a, const Team &t, PatchSmem &ps, unsigned int G,
                                                   unsigned long long mx_bits, unsigned int value) {
  // sweep G - 1's word, read ahead for lag_decide: its load overlaps the reduction and the fence
  unsigned long long pre = 0ull;
  if (threadIdx.x == 0 && G > 0u)
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(pre) : "l"(&a.ctl->lag_word[(G - 1u) % kLagRing]) : "memory");
  const unsigned long long x = block_max_u64(mx_bits);
  if (threadIdx.x == 0) {
    ps.lag_pre = pre;
    ps.lag_pre_g = G - 1u;
    unsigned long long key;
    const unsigned long long inc = lag_increment(x, a.tol, G, &key);
    atomicMax(&a.ctl->lag_res[G % kLagRing], key);
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(&a.ctl->lag_word[G % kLagRing]), "l"(inc) : "memory");
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(a.prog + 32 * t.rank()), "r"(value) : "memory");
  }
}

// The decision on sweep G for the whole block: 1 converged, 2 diverged, 0 neither, -1 when a
// bounded wait ran out, the team's error bit is set, or the slot was refilled early.
template <class Team>
__device__ __forceinline__ int lag_decide(const SsaArgs &a, const Team &t, PatchSmem &ps, unsigned int G) {
  if (threadIdx.x == 0) {
    const unsigned int slot = G % kLagRing;
    const unsigned long long *wp = &a.ctl->lag_word[slot];
    const unsigned long long n = (unsigned long long)t.size();
    const unsigned long long prev = ps.lag_prev[slot];
    unsigned long long d = 0ull;
    bool have = false;   // the word read ahead holds the whole sweep
    if (ps.lag_pre_g == G) {
      d = ps.lag_pre - prev;
      have = (d & 0xffffull) == n;
    }
    if (!have) d = ld_acquire_u64(wp) - prev;
    int act = 0;
    if ((d & 0xffffull) < n) {
      const unsigned long long t0 = globaltimer_ns();
      unsigned int ns = 16;
      for (;;) {
        __nanosleep(ns);
        if (ns < 64) ns <<= 1;
        d = ld_acquire_u64(wp) - prev;
        if ((d & 0xffffull) >= n) break;
        if (*(volatile unsigned int *)t.bar() & kBarrierError) { act = -1; break; }
        if ((long long)(globaltimer_ns() - t0) > a.timeout_ns) {
          atomicCAS(&a.ctl->err, 0, (int)UFE_TIMEOUT);
          atomicOr(t.bar(), kBarrierError);
          act = -1;
          break;
        }
      }
    }
    if (act == 0 && (d & 0xffffull) != n) {
      atomicCAS(&a.ctl->err, 0, (int)UFE_TIMEOUT);
      atomicOr(t.bar(), kBarrierError);
      act = -1;
    }
    if (act == 0) {
      ps.lag_prev[slot] = prev + d;
      const unsigned int nc = (unsigned int)(d >> 16) & 0xffffu, nd = (unsigned int)(d >> 32) & 0xffffu;
      const unsigned int nn = (unsigned int)(d >> 48);
      act = nn ? 0 : nc == 0 ? 1 : nd ? 2 : 0;
    }
    ps.lag_act[G & 1] = act;   // two cells: a fast thread 0 may write the next sweep's before all read this one
  }
  __syncthreads();
  return ps.lag_act[G & 1];
}

// The final maximum |res| of sweep G (the report), read by thread 0 after lag_decide took G.
__device__ __forceinline__ double lag_residual_of(const SsaArgs &a, unsigned int G) {
  const unsigned long long key = *(volatile unsigned long long *)&a.ctl->lag_res[G % kLagRing];
  return (unsigned int)(key >> 32) == G + 1u ? (double)__uint_as_float((unsigned int)key) : -1.0;
}

// End of a linear solve with lagged decisions: the sweeps after the deciding one (`decided`)
// are read without acting, so that every CTA has read every sweep of its slots; the leader
// takes the deciding sweep's maximum |res| for the report.
template <class Team>
__device__ __forceinline__ bool lag_drain(const SsaArgs &a, const Team &t, PatchSmem &ps, unsigned int base,
                                          int decided, int sweeps, bool leader, double &maxres) {
  const int last = decided;
  while (decided < sweeps) {
    ++decided;
    if (lag_decide(a, t, ps, base + (unsigned)(decided - 1)) < 0) {
      if (threadIdx.x == 0) a.prog[32 * t.rank()] = 0x7fffffffu;
      return false;
    }
  }
  if (leader && last > 0) maxres = lag_residual_of(a, base + (unsigned)(last - 1));
  return true;
}

// Patch b's slice table, edge range and synchronisation set into shared memory.
template <class Args>
__device__ __forceinline__ void load_patch(const Args &a, int b, PatchSmem &ps) {
  if (threadIdx.x < 8) ps.lag_prev[threadIdx.x] = 0ull;
  if (threadIdx.x == 0) ps.lag_pre_g = 0xffffffffu;   // nothing read ahead (lag_decide)
  if (threadIdx.x <= kGroups) ps.ps[threadIdx.x] = a.patch_slice[b * (kGroups + 1) + threadIdx.x];
  if (threadIdx.x == 0) {
    ps.edge0 = a.patch_edge0[b];
    ps.edge1 = a.patch_edge0[b + 1];
    ps.nsync = a.sync_ptr[b + 1] - a.sync_ptr[b];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ps.nsync; i += blockDim.x) ps.sync[i] = a.sync_list[a.sync_ptr[b] + i];
  for (int s = ps.ps[0] + threadIdx.x; s < ps.ps[kGroups]; s += blockDim.x) {
    ps.e0[s - ps.ps[0]] = a.slice_e0[s];
    ps.w[s - ps.ps[0]] = a.slice_w[s];
  }
  __syncthreads();
}

// Patch b's halo program (phase slice ranges and slice table), own rows, halo slots and the
// patches of its start-of-sweep wait into shared memory.
__device__ __forceinline__ void load_patch_halo(const SsaArgs &a, int b, PatchSmem &ps) {
  if (threadIdx.x < 8) ps.lag_prev[threadIdx.x] = 0ull;
  if (threadIdx.x == 0) ps.lag_pre_g = 0xffffffffu;
  if (threadIdx.x <= kGroups) ps.ps[threadIdx.x] = a.patch_slice[b * (kGroups + 1) + threadIdx.x];
  if (threadIdx.x < 8) ps.hps[threadIdx.x] = a.hp_slice[b * 7 + threadIdx.x];
  if (threadIdx.x == 0) {
    ps.nsync = a.hsync_ptr[b + 1] - a.hsync_ptr[b];
    ps.hsplit = a.hp_split[b];
    ps.hl0 = a.hload_ptr[b];
    ps.nh = a.hload_ptr[b + 1] - a.hload_ptr[b];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ps.p0 = ps.ps[0] * kSlice;
    ps.n_own = (ps.ps[kGroups] - ps.ps[0]) * kSlice;
  }
  for (int i = threadIdx.x; i < ps.nsync; i += blockDim.x) ps.sync[i] = a.hsync_list[a.hsync_ptr[b] + i];
  for (int s = ps.hps[0] + threadIdx.x; s < ps.hps[7]; s += blockDim.x) {
    ps.e0[s - ps.hps[0]] = a.hslice_e0[s];
    ps.w[s - ps.hps[0]] = a.hslice_w[s];
  }
  __syncthreads();
}

// The whole solve_SSA of one problem, run by the CTAs of a team (each CTA owns one patch).
// Returns false when a bounded wait failed; the error is recorded in the problem's control
// block and the team's barrier counter. kHalo: the halo sweeps (one neighbour wait per
// sweep, the patch's working copy in shared memory, velocities in three buffers by sweep).
template <int kMode, class Team, bool kHalo = false>
__device__ bool solve_member(const SsaArgs &a, Team &t) {
  constexpr bool kM = kMode == kMixed;
  using T = typename std::conditional<kM, float2, double2>::type;
  SsaCtl *ctl = a.ctl;
  unsigned int phases = 0;   // colour phases (halo sweeps: sweeps) completed by this patch
  const bool leader = t.rank() == 0 && threadIdx.x == 0;
  __shared__ PatchSmem ps;
  if constexpr (kHalo) load_patch_halo(a, t.rank(), ps);
  else load_patch(a, t.rank(), ps);
  extern __shared__ __align__(16) unsigned char ufe_local_rows[];
  const LocalRows lc{ufe_local_rows, ps.ps[0] * kSlice,
                     (kMode != kExact64 && a.local_rows) ? (ps.ps[kGroups] - ps.ps[0]) * kSlice : 0};
  T *const hbuf0 = reinterpret_cast<T *>(kM ? (void *)a.dUV : (void *)a.UV);
  T *const hbuf1 = reinterpret_cast<T *>(kM ? (void *)a.dUVb : (void *)a.UVb);
  T *const hbuf2 = reinterpret_cast<T *>(kM ? (void *)a.dUVc : (void *)a.UVc);
  T *const hld = reinterpret_cast<T *>(ufe_local_rows);
  int *const hidx = reinterpret_cast<int *>(ufe_local_rows + (size_t)a.halo_index_off);
  unsigned char *const hstage = ufe_local_rows + (size_t)a.stage_off;
  if constexpr (kHalo) {
    for (int i = threadIdx.x; i < ps.nh; i += blockDim.x) hidx[i] = a.hload_dev[ps.hl0 + i];
    __syncthreads();
    if constexpr (kM) halo_stage(a, ps, hstage);
  }
  // (Re)load the mirror from global memory: at the start and after the grid-wide phases
  // that rewrite every row (fold, reset). Halo sweeps: the own rows of the working copy, also
  // copied into the other two buffers, which then hold every row that no sweep writes
  // (Dirichlet rows) as well.
  auto reload = [&]() {
    if constexpr (kHalo) {
      for (int i = threadIdx.x; i < ps.n_own; i += blockDim.x) {
        const T v = hbuf0[ps.p0 + i];
        hld[i] = v;
        hbuf1[ps.p0 + i] = v;
        hbuf2[ps.p0 + i] = v;
      }
      __syncthreads();
      return;
    }
    if (!lc.n) return;
    for (int i = threadIdx.x; i < lc.n; i += blockDim.x) {
      if (kM) static_cast<float2 *>(lc.base)[i] = a.dUV[lc.p0 + i];
      else static_cast<double2 *>(lc.base)[i] = a.UV[lc.p0 + i];
    }
    __syncthreads();
  };
  reload();
  double *N = a.Na, *Nprev = a.Nb;
  int did_reset_before = 0;
  int it = 0;
  unsigned int gsweep = 0;   // sweeps of this launch (the lagged decisions' ring index)
  bool picard_done = false;
  UFE_TM_DECL
#define UFE_GRID_SYNC()                                   \
  if (!team_barrier(t, &ctl->err, a.timeout_ns)) {        \
    if (threadIdx.x == 0) a.prog[32 * t.rank()] = 0x7fffffffu; \
    return false;                                         \
  }
  while (!picard_done && it < a.max_outer) {
    ++it;
    // N_prev <- N, then the new viscosity into N
    { double *t = N; N = Nprev; Nprev = t; }
    phase_viscosity(a, t, N, Nprev, kM && a.fp32_visc);
    UFE_GRID_SYNC();
    const double RN = final_rn(a, t);
    if (leader) { ctl->picard_iterations = it; ctl->last_RN = RN; }
    if (RN < a.rn_tol) { picard_done = true; break; }
    phase_coefficients<kMode>(a, t);
    if (leader) { ctl->maxres[0] = 0ull; ctl->maxres[1] = 0ull; ctl->maxres[2] = 0ull; }
    UFE_GRID_SYNC();
    if (kM) {
      phase_defect(a, t);
      UFE_GRID_SYNC();
    }
    // Coloured SOR. Colour phases synchronise only with the neighbouring patches; the
    // boundary phase ends with a grid barrier, after which the sweep's maximum residual is
    // known to every CTA.
    int sweeps = 0;
    bool lin_done = false;
    int did_reset = 0;
    double maxres = 0.0;
    if constexpr (kHalo) {
      // Halo sweeps. Every patch's rows of a sweep go to the next of three buffers (cur: the one
      // holding the latest rows). A sweep first runs colour 1's own rows that read no halo slot
      // (their inputs are own rows of the working copy; the buffer it writes was last read by
      // the neighbouring patches two sweeps ago, before they completed the sweep this patch
      // waited for at the start of the previous one), then waits once for the patches whose rows
      // it reads and that read its rows (they finished the previous sweep, so buffer cur holds
      // their rows), loads its halo slots, and runs the rest of the seven phases on its working
      // copy with CTA barriers only. Sync points commit the own rows to the canonical buffer.
      constexpr bool kLag = kM && kMixedLag > 0;
      auto hb = [&](int i) { return i == 0 ? hbuf0 : i == 1 ? hbuf1 : hbuf2; };
      int cur = 0;
      bool synced = true;
      int decided = 0;
      const unsigned int base = gsweep;
      halo_refresh<kMode>(a, ps, hstage);
      UFE_TM(kTmOther);
      while (!lin_done && sweeps < a.max_inner) {
        ++sweeps;
        UFE_TM_COUNT(kTmSweeps);
        const unsigned int G = gsweep++;
        const int slot = sweeps % 3;
        if (!kLag && leader) ctl->maxres[(sweeps + 1) % 3] = 0ull;
        T *const out = hb(cur == 2 ? 0 : cur + 1);
        auto colour = [&](int s_begin, int s_end, int nw) -> unsigned long long {
          if constexpr (kM) return halo_colour32(a, ps, s_begin, s_end, nw, hstage, hidx, hld, out);
          else return halo_colour64<kMode == kExact64>(a, ps, s_begin, s_end, nw, hld, out);
        };
        // the last kFetchWarps warps wait for the neighbouring patches and load the halo slots
        // while the others run colour 1's halo-free rows
        // (the FP64 modes, with a team barrier after every sweep, wait for nothing here and run
        // colour 1 whole)
        const int nwarps = blockDim.x >> 5;
        unsigned long long mx = 0ull;
        if constexpr (kLag) {
          if ((int)(threadIdx.x >> 5) < nwarps - kFetchWarps) mx = colour(ps.hps[0], ps.hsplit, nwarps - kFetchWarps);
          else halo_fetch(a, ps, phases, t.bar(), !synced, hidx, hld, hb(cur));
        } else {
          halo_load(ps, hidx, hld, hb(cur));
        }
        __syncthreads();
        UFE_TM(kTmWaitColour);
        for (int f = 0; f < 5; ++f) {
          const int s_begin = f == 0 && kLag ? ps.hsplit : ps.hps[f];
          if (ps.hps[f + 1] == s_begin) continue;
          const unsigned long long m = colour(s_begin, ps.hps[f + 1], nwarps);
          mx = m > mx ? m : mx;
          __syncthreads();
          UFE_TM_SUB(kTmColour0 + f);
        }
        UFE_TM(kTmColour);
        for (int f = 5; f < 7; ++f) {
          if (ps.hps[f + 1] == ps.hps[f]) continue;
          halo_boundary<kM>(a, ps, f, hld, out);
          __syncthreads();
        }
        UFE_TM(kTmBoundary);
        cur = cur == 2 ? 0 : cur + 1;
        if constexpr (kLag) {
          ++phases;
          lag_arrive_publish(a, t, ps, G, mx, phases);
          UFE_TM(kTmArrive);
          synced = false;
          const bool refold_now = a.refold > 0 && sweeps % a.refold == 0;
          const bool sync_point = sweeps == a.max_inner || refold_now;
          if (sync_point) {
            if (cur) halo_store_own(ps, hld, hbuf0);
            cur = 0;
            UFE_GRID_SYNC();
            synced = true;
            UFE_TM(kTmGrid);
          }
          const int upto = sync_point ? sweeps : sweeps - kMixedLag;
          int act = 0;             // 1: converged, 2: diverged
          while (decided < upto && act == 0) {
            ++decided;
            act = lag_decide(a, t, ps, base + (unsigned)(decided - 1));
            if (act < 0) {
              if (threadIdx.x == 0) a.prog[32 * t.rank()] = 0x7fffffffu;
              return false;
            }
          }
          UFE_TM(kTmDecide);
          if (act == 1) {
            lin_done = true;
          } else if (act == 2) {
            if (!synced) { UFE_GRID_SYNC(); synced = true; }
            phase_zero_velocity(a, t, kM);
            UFE_GRID_SYNC();
            reload();
            cur = 0;
            did_reset = 1;
            lin_done = true;
          } else if (sweeps == a.max_inner) {
            if (leader) ctl->not_converged += 1;
          } else if (refold_now) {
            phase_fold(a, t);
            UFE_GRID_SYNC();
            reload();
            phase_defect(a, t);
            UFE_GRID_SYNC();
            halo_refresh<kMode>(a, ps, hstage);
          }
          UFE_TM(kTmOther);
        } else {
          block_max_to(&ctl->maxres[slot], mx);
          UFE_TM(kTmArrive);
          UFE_GRID_SYNC();
          UFE_TM(kTmGrid);
          maxres = __longlong_as_double((long long)*(volatile unsigned long long *)&ctl->maxres[slot]);
          if (maxres < a.tol) {
            lin_done = true;
          } else if (maxres > 1e6) {
            phase_zero_velocity(a, t, kM);
            UFE_GRID_SYNC();
            reload();
            cur = 0;
            did_reset = 1;
            lin_done = true;
          } else if (sweeps == a.max_inner) {
            if (leader) ctl->not_converged += 1;
          } else if (kM && a.refold > 0 && sweeps % a.refold == 0) {
            if (cur) halo_store_own(ps, hld, hbuf0);
            cur = 0;
            UFE_GRID_SYNC();
            phase_fold(a, t);
            UFE_GRID_SYNC();
            reload();
            phase_defect(a, t);
            UFE_GRID_SYNC();
            halo_refresh<kMode>(a, ps, hstage);
          }
          UFE_TM(kTmOther);
        }
      }
      if constexpr (kLag) {
        if (!lag_drain(a, t, ps, base, decided, sweeps, leader, maxres)) return false;
      }
      // the final own rows into the canonical buffer before the grid-wide phases read it
      const bool commit = cur || (kLag && !synced);
      if (cur) halo_store_own(ps, hld, hbuf0);
      if (commit) UFE_GRID_SYNC();
      UFE_TM(kTmGrid);
    } else
    if constexpr (kM && kMixedLag > 0) {
      // Mixed sweeps with lagged decisions: the boundary phase is a counted phase and the next
      // sweep's first colour waits for the neighbours' boundary rows, so no team barrier
      // separates sweeps; sweep j's residual decides at the end of sweep j + lag (every CTA
      // reads the same value, so every CTA takes the same decision and does the same
      // sweeps). Refolds and the last allowed sweep are barriers, where the sweeps not yet
      // decided are decided in order.
      bool synced = true;        // a team barrier follows the previous phases of this CTA
      int decided = 0;           // sweeps of this linear solve already decided
      const unsigned int base = gsweep;
      UFE_TM(kTmOther);
      while (!lin_done && sweeps < a.max_inner) {
        ++sweeps;
        UFE_TM_COUNT(kTmSweeps);
        const unsigned int G = gsweep++;
        unsigned long long mx = 0ull;
        for (int g = 0; g < 5; ++g) {
          if (g > 0 || !synced) wait_neighbours(a, ps, phases, t.bar());
          UFE_TM(kTmWaitColour);
          const unsigned long long m = phase_sweep32(a, ps, g, lc);
          mx = m > mx ? m : mx;
          ++phases;
          publish_progress(a, t, phases);
          UFE_TM(kTmColour);
        }
        lag_arrive(a, G, mx);
        UFE_TM(kTmArrive);
        wait_neighbours(a, ps, phases, t.bar());
        UFE_TM(kTmWaitBoundary);
        phase_boundary<kM>(a, ps, lc);
        ++phases;
        publish_progress(a, t, phases);
        UFE_TM(kTmBoundary);
        synced = false;
        const bool refold_now = a.refold > 0 && sweeps % a.refold == 0;
        const bool sync_point = sweeps == a.max_inner || refold_now;
        if (sync_point) {
          UFE_GRID_SYNC();
          synced = true;
          UFE_TM(kTmGrid);
        }
        const int upto = sync_point ? sweeps : sweeps - kMixedLag;
        int act = 0;             // 1: converged, 2: diverged
        while (decided < upto && act == 0) {
          ++decided;
          act = lag_decide(a, t, ps, base + (unsigned)(decided - 1));
          if (act < 0) {
            if (threadIdx.x == 0) a.prog[32 * t.rank()] = 0x7fffffffu;
            return false;
          }
        }
        UFE_TM(kTmDecide);
        if (act == 1) {
          lin_done = true;
        } else if (act == 2) {
          if (!synced) { UFE_GRID_SYNC(); synced = true; }
          phase_zero_velocity(a, t, kM);
          UFE_GRID_SYNC();
          reload();
          did_reset = 1;
          lin_done = true;
        } else if (sweeps == a.max_inner) {
          if (leader) ctl->not_converged += 1;
        } else if (refold_now) {
          phase_fold(a, t);
          UFE_GRID_SYNC();
          reload();
          phase_defect(a, t);
          UFE_GRID_SYNC();
        }
        UFE_TM(kTmOther);
      }
      if (!lag_drain(a, t, ps, base, decided, sweeps, leader, maxres)) return false;
      if (!synced) UFE_GRID_SYNC();
      UFE_TM(kTmGrid);
    } else
    while (!lin_done && sweeps < a.max_inner) {
      ++sweeps;
      UFE_TM(kTmOther);
      UFE_TM_COUNT(kTmSweeps);
      const int slot = sweeps % 3;
      if (leader) ctl->maxres[(sweeps + 1) % 3] = 0ull;
      unsigned long long mx = 0ull;
      for (int g = 0; g < 5; ++g) {
        if (g > 0) wait_neighbours(a, ps, phases, t.bar());
        UFE_TM(kTmWaitColour);
        unsigned long long m;
        if (kMode == kExact64) m = phase_sweep_exact(a, ps, g);
        else if (kMode == kFast64) m = phase_sweep_fast(a, ps, g, lc);
        else m = phase_sweep32(a, ps, g, lc);
        mx = m > mx ? m : mx;
        ++phases;
        publish_progress(a, t, phases);
        UFE_TM(kTmColour);
      }
      block_max_to(&ctl->maxres[slot], mx);
      UFE_TM(kTmArrive);
      wait_neighbours(a, ps, phases, t.bar());
      UFE_TM(kTmWaitBoundary);
      phase_boundary<kM>(a, ps, lc);
      UFE_TM(kTmBoundary);
      UFE_GRID_SYNC();
      UFE_TM(kTmGrid);
      maxres = __longlong_as_double((long long)*(volatile unsigned long long *)&ctl->maxres[slot]);
      if (maxres < a.tol) {
        lin_done = true;
      } else if (maxres > 1e6) {
        phase_zero_velocity(a, t, kM);
        UFE_GRID_SYNC();
        reload();
        did_reset = 1;
        lin_done = true;
      } else if (sweeps == a.max_inner) {
        if (leader) ctl->not_converged += 1;
      } else if (kM && a.refold > 0 && sweeps % a.refold == 0) {
        phase_fold(a, t);
        UFE_GRID_SYNC();
        reload();
        phase_defect(a, t);
        UFE_GRID_SYNC();
      }
    }
    if (kM && !did_reset) {
      phase_fold(a, t);
      UFE_GRID_SYNC();
      reload();
    }
    if (leader) {
      if (ctl->linear_solves < 64) ctl->sweeps[ctl->linear_solves] = sweeps;
      ctl->linear_solves += 1;
      ctl->total_sweeps += sweeps;
      ctl->last_max_residual = maxres;
      if (did_reset) ctl->resets += 1;
    }
    if (did_reset) {
      if (did_reset_before) {
        if (leader) ctl->status = UFE_DIVERGED;
        break;
      }
      did_reset_before = 1;
    }
  }
  // Final N lives in N; make Na hold it for the scatter.
  if (N != a.Na) {
    const int tid = t.rank() * blockDim.x + threadIdx.x;
    const int nt = t.size() * blockDim.x;
    UFE_GRID_SYNC();
    for (int p = tid; p < a.nP; p += nt) a.Na[p] = N[p];
  }
  UFE_GRID_SYNC();
  UFE_TM(kTmOther);
  UFE_TM_FLUSH();
  return true;
#undef UFE_GRID_SYNC
}

// Stage the argument block in shared memory (it is read on every phase by every thread).
__device__ __forceinline__ void stage_args(SsaArgs &dst, const SsaArgs *src) {
  const int n = (int)(sizeof(SsaArgs) / sizeof(int));
  int *d = reinterpret_cast<int *>(&dst);
  const int *q = reinterpret_cast<const int *>(src);
  for (int i = threadIdx.x; i < n; i += blockDim.x) d[i] = q[i];
  __syncthreads();
}

// Single solve: the whole grid is one team; the argument block stays in the kernel's
// parameter space (constant bank operands cost no registers).
template <int kMode, bool kHalo>
__global__ void __launch_bounds__(kHalo ? kHaloBlock : kSsaBlock, kCtasPerSm) ssa_persistent(const SsaArgs a) {
  GridTeam t{&a.ctl->bar_count, 0u};
  solve_member<kMode, GridTeam, kHalo>(a, t);
}

// Ensemble of independent solves in one launch. The grid is cut into teams; a team of T
// CTAs solves members whose meshes have T patches. Teams of one size form a class with
// its own queue (members ordered by expected cost, largest first); each team takes the
// next member of its class until the queue is empty.
struct BatchArgs {
  const SsaArgs *members;        // [n_members] grouped by class, device
  int n_members;
  const int *team_of_cta;        // [grid]
  const int4 *team_info;         // [n_teams] (first CTA, CTAs, class, -)
  const int2 *class_range;       // [n_classes] queue positions [begin, end) in members
  unsigned int *queue;           // [n_classes * 32] next position of each class (offset from begin)
  unsigned int *team_bar;        // [n_teams * 32] barrier counters
  unsigned int *team_member;     // [n_teams * 32] position being solved
  unsigned long long *times;     // [n_members * 2] start / end (globaltimer ns) by position
  int *err;                      // first failure of any team
  long long timeout_ns;
};

// kHalo (mixed only): the members run the halo sweeps (every member has the program).
template <int kMode, int kBlock, int kPerSm, bool kHalo = false>
__global__ void __launch_bounds__(kBlock, kPerSm) ssa_batched(const BatchArgs b) {
  __shared__ SsaArgs a;
  const int team = b.team_of_cta[blockIdx.x];
  const int4 ti = b.team_info[team];
  SubTeam t{(int)blockIdx.x - ti.x, ti.y, b.team_bar + 32 * team, 0u};
  const int2 cr = b.class_range[ti.z];
  for (;;) {
    if (t.rank() == 0 && threadIdx.x == 0) {
      unsigned int m = (unsigned)cr.x + atomicAdd(b.queue + 32 * ti.z, 1u);
      if (m >= (unsigned)cr.y) m = 0xffffffffu;
      b.team_member[32 * team] = m;
      if (m < (unsigned)b.n_members) b.times[2 * m] = globaltimer_ns();
    }
    if (!team_barrier(t, b.err, b.timeout_ns)) return;
    const unsigned int m = *(volatile unsigned int *)&b.team_member[32 * team];
    if (m >= (unsigned)b.n_members) return;
    stage_args(a, b.members + m);
    if (!solve_member<kMode, SubTeam, kHalo>(a, t)) {
      if (threadIdx.x == 0) atomicCAS(b.err, 0, (int)UFE_TIMEOUT);
      return;
    }
    if (t.rank() == 0 && threadIdx.x == 0) b.times[2 * m + 1] = globaltimer_ns();
  }
}

// ---------------------------------------------------------------------------------------
// Adjoint of the converged solve (no counterpart in the reference)
//
// F(u) = 0 is the discrete system the Picard/SOR loop converges to: on interior rows the
// momentum balance with eta = eta(u) (and the friction factor S / (max(0.1, H) eta) on
// grounded rows), on edge rows the Neumann averages. The VJP solves (dF/du)^T mu = dJ/du by
// a transposed coloured SOR: per sweep the corners, the other edge rows, then colours 5..1
// (the reverse of the forward's block order, which makes the transposed iteration converge
// like the forward one). Transposed row j gathers over its neighbours i the coefficients of
// u_j in equation i: Cu_ij mu_x,i + kU_ij s_i, with s_i = alpha_x,i mu_x,i + alpha_y,i mu_y,i
// the linearised viscosity of row i (eta' lumped per row) and kU_ij the strain-rate
// derivative d(eps^2)/dU_j through row i's neighbour functions; for an edge or corner
// neighbour i the coefficient is its averaging weight.
// ---------------------------------------------------------------------------------------
struct AdjCtl {
  unsigned int bar_count;         // monotonic grid-barrier counter (bit 30: error)
  int err;
  int status;
  int sweeps;
  unsigned long long maxd[3];     // max |update| per sweep (ring), ordered bits
  unsigned long long maxm[3];     // max |mu| per sweep (ring)
  double last_rel;
  int not_found;                  // transposed entries without a reverse entry (asymmetric mesh)
  int pad_;
};

struct AdjArgs {
  const int *col;
  const uint8_t *deg;
  const int *orig_of_dev;
  const int *slice_e0;
  const uint8_t *slice_w;
  const int *patch_slice;
  const int *patch_edge0;
  const int *sync_ptr;
  const int *sync_list;
  unsigned int *prog;
  const double2 *cT, *kT;   // [nE] transposed coefficients
  const double2 *ee;        // [nP] (eu, ev) on interior rows
  const double *c3;         // [nP] 3 sNxy
  const double2 *kh;        // [nP] home strain derivatives (kU_ii, kV_ii)
  const double2 *alpha;     // [nP]
  const double2 *dinv;      // [nP] 1 / transposed diagonal
  const double2 *g;         // [nP] dJ/du
  double2 *mu;
  double *s;
  AdjCtl *ctl;
  double omega, tol;
  int max_sweeps;
  long long timeout_ns;
};

// One phase of the transposed sweep over group g of the patch. kind 0: interior rows of a
// colour (SOR update); 1: the corners, 2: the other edge rows (exact update, unit diagonal).
__device__ void adj_phase(const AdjArgs &a, const PatchSmem &ps, int g, int kind, unsigned long long &mxd,
                          unsigned long long &mxm) {
  const int wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (int s = ps.ps[g] + wid; s < ps.ps[g + 1]; s += nwarps) {
    const int w = ps.w[s - ps.ps[0]];
    const int64_t e0 = ps.e0[s - ps.ps[0]] + lane;
    const int p = s * kSlice + lane;
    if (a.deg[p] == 0) continue;
    if (kind != 0 && ((kind == 1) != (a.orig_of_dev[p] < 4))) continue;
    double rx = 0.0, ry = 0.0;
    for (int k = 0; k < w; ++k) {
      const int64_t e = e0 + (int64_t)k * kSlice;
      const int j = a.col[e];
      if (j < 0) break;
      const double2 c = a.cT[e];
      const double2 kk = a.kT[e];
      const double2 m = a.mu[j];
      const double sj = a.s[j];
      rx = fma(c.x, m.x, fma(kk.x, sj, rx));
      ry = fma(c.y, m.y, fma(kk.y, sj, ry));
    }
    const double2 mi = a.mu[p];
    const double2 gi = a.g[p];
    double dx, dy;
    if (kind == 0) {
      const double2 ec = a.ee[p];
      const double c3 = a.c3[p];
      const double2 kh = a.kh[p];
      const double sp = a.s[p];
      rx = fma(ec.x, mi.x, fma(c3, mi.y, fma(kh.x, sp, rx))) - gi.x;
      ry = fma(ec.y, mi.y, fma(c3, mi.x, fma(kh.y, sp, ry))) - gi.y;
      const double2 di = a.dinv[p];
      dx = -a.omega * rx * di.x;
      dy = -a.omega * ry * di.y;
    } else {
      dx = -(rx + mi.x - gi.x);
      dy = -(ry + mi.y - gi.y);
    }
    const double2 mn = make_double2(mi.x + dx, mi.y + dy);
    a.mu[p] = mn;
    if (kind == 0) {
      const double2 al = a.alpha[p];
      a.s[p] = fma(al.x, mn.x, al.y * mn.y);
    }
    unsigned long long b = abs_bits(dx);
    mxd = b > mxd ? b : mxd;
    b = abs_bits(dy);
    mxd = b > mxd ? b : mxd;
    b = abs_bits(mn.x);
    mxm = b > mxm ? b : mxm;
    b = abs_bits(mn.y);
    mxm = b > mxm ? b : mxm;
  }
}

__global__ void __launch_bounds__(kSsaBlock, kCtasPerSm) ssa_adjoint_sor(const AdjArgs a) {
  GridTeam t{&a.ctl->bar_count, 0u};
  AdjCtl *ctl = a.ctl;
  __shared__ PatchSmem ps;
  load_patch(a, t.rank(), ps);
  const bool leader = t.rank() == 0 && threadIdx.x == 0;
  unsigned int phases = 0;
  int sweeps = 0;
  for (;;) {
    ++sweeps;
    const int slot = sweeps % 3;
    if (leader) { ctl->maxd[(sweeps + 1) % 3] = 0ull; ctl->maxm[(sweeps + 1) % 3] = 0ull; }
    unsigned long long mxd = 0ull, mxm = 0ull;
    for (int ph = 0; ph < 7; ++ph) {
      if (ph > 0) wait_neighbours(a, ps, phases, t.bar());
      if (ph == 0) adj_phase(a, ps, 5, 1, mxd, mxm);
      else if (ph == 1) adj_phase(a, ps, 5, 2, mxd, mxm);
      else adj_phase(a, ps, 6 - ph, 0, mxd, mxm);   // colours 5, 4, 3, 2, 1
      ++phases;
      publish_progress(a, t, phases);
    }
    block_max_to(&ctl->maxd[slot], mxd);
    block_max_to(&ctl->maxm[slot], mxm);
    if (!team_barrier(t, &ctl->err, a.timeout_ns)) {
      if (threadIdx.x == 0) a.prog[32 * t.rank()] = 0x7fffffffu;
      return;
    }
    const double md = __longlong_as_double((long long)*(volatile unsigned long long *)&ctl->maxd[slot]);
    const double mm = __longlong_as_double((long long)*(volatile unsigned long long *)&ctl->maxm[slot]);
    // A non-finite update or state (NaN bits order above infinity) means the iteration
    // diverged (possible for relaxation factors well above the forward's).
    if (!isfinite(md) || !isfinite(mm)) {
      if (leader) { ctl->sweeps = sweeps; ctl->last_rel = md; ctl->status = UFE_DIVERGED; }
      return;
    }
    const double rel = mm > 0.0 ? md / mm : 0.0;
    if (rel < a.tol || sweeps >= a.max_sweeps) {
      if (leader) {
        ctl->sweeps = sweeps;
        ctl->last_rel = rel;
        ctl->status = rel < a.tol ? UFE_OK : UFE_NOT_CONVERGED;
      }
      return;
    }
  }
}

// ---- Krylov acceleration of the transposed SOR (GMRES on the sweep's fixed-point map) ----
// One transposed sweep maps mu to S(mu; g) = G mu + M^-1 g. GMRES solves (I - G) mu = S(0; g)
// with the operator x -> x - S(x; 0): one sweep per Krylov iteration, left-preconditioned by
// the sweep itself. Vectors are the (mu_x, mu_y) pairs of the nP device rows.
__global__ void k_krylov_load(int nP, const double2 *x, const double2 *alpha, double2 *mu, double *s) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nP) return;
  const double2 v = x ? x[p] : make_double2(0.0, 0.0);
  const double2 al = alpha[p];
  mu[p] = v;
  s[p] = fma(al.x, v.x, al.y * v.y);
}

// y = x - mu
__global__ void k_krylov_sub(int n, const double *x, const double *mu, double *y) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) y[e] = x[e] - mu[e];
}

// Block partial sums of V_i . w: part[i * gridDim.x + block], i = blockIdx.y.
__global__ void k_krylov_dots(int n, const double *V, size_t ld, const double *w, double *part) {
  const double *v = V + (size_t)blockIdx.y * ld;
  double acc = 0.0;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) acc = fma(v[e], w[e], acc);
  __shared__ double sw[32];
  acc = warp_sum(acc);
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sw[wid] = acc;
  __syncthreads();
  if (wid == 0) {
    double x = lane < (int)(blockDim.x >> 5) ? sw[lane] : 0.0;
    x = warp_sum(x);
    if (lane == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = x;
  }
}

// w -= sum_i h_i V_i (i < nvec)
__global__ void k_krylov_axpy(int n, int nvec, const double *V, size_t ld, const double *h, double *w) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double acc = 0.0;
  for (int i = 0; i < nvec; ++i) acc = fma(h[i], V[(size_t)i * ld + e], acc);
  w[e] = w[e] - acc;
}

__global__ void k_krylov_scale(int n, const double *w, double f, double *v) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) v[e] = w[e] * f;
}

// Per-row set-up of the adjoint operator at the converged velocities: strain rates,
// viscosity, friction factor, the linearised-viscosity weights alpha and the transposed
// diagonal. Boundary rows get unit diagonals and no viscosity term.
struct AdjSetup {
  int nP, nV;
  const int *col;
  const uint8_t *deg;
  const int *slice_e0;
  const uint8_t *slice_g;
  const int *orig_of_dev;
  const double2 *nxy, *h_nxy, *h_cuv;
  const double *sNxy;
  const double *Hi, *Hb, *SL, *hx, *hy, *Af, *beta;
  const double *tau;                           // Coulomb_regularised: the solve's basal yield stress
  double beta_const, m_enh;
  int coulomb;                                 // 1: Coulomb_regularised law, 0: linear (S = beta^2)
  double uq, expo;                             // Coulomb: u_threshold^q and (q - 1) / 2
  const double2 *UV;
  const double *dJ_U, *dJ_V, *dJ_Ux, *dJ_Uy;   // caller order, staged on the device
  double2 *ee, *kh, *alpha, *dinv, *g, *mu;
  double *c3, *s, *eta, *fr, *inv_nb;
  double *K;                                   // [3 nP] strain combinations 2ux+vy, (uy+vx)/2, 2vy+ux
  double omega;
};

__device__ __forceinline__ int64_t sell_entry(const int *slice_e0, int p, int k) {
  return (int64_t)slice_e0[p / kSlice] + (int64_t)k * kSlice + (p % kSlice);
}

__global__ void k_adj_rows(const AdjSetup a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.nP) return;
  const int n = a.deg[p];
  const int r = a.orig_of_dev[p];
  a.mu[p] = make_double2(0.0, 0.0);
  a.s[p] = 0.0;
  if (n == 0 || r < 0) {
    a.ee[p] = make_double2(1.0, 1.0); a.kh[p] = make_double2(0.0, 0.0); a.alpha[p] = make_double2(0.0, 0.0);
    a.dinv[p] = make_double2(1.0, 1.0); a.g[p] = make_double2(0.0, 0.0); a.c3[p] = 0.0;
    a.eta[p] = 1.0; a.fr[p] = 0.0; a.inv_nb[p] = 0.0;
    a.K[p] = 0.0; a.K[a.nP + p] = 0.0; a.K[2 * a.nP + p] = 0.0;
    return;
  }
  a.g[p] = r < a.nV ? make_double2(a.dJ_U[r], a.dJ_V[r]) : make_double2(a.dJ_Ux[r - a.nV], a.dJ_Uy[r - a.nV]);
  const bool edge = a.slice_g[p / kSlice] == 5;
  const bool corner = r < 4;
  // strain rates (get_mesh_derivatives_AaAc, home term first)
  const double2 ui = a.UV[p];
  const double2 hn = a.h_nxy[p];
  double ux = hn.x * ui.x, uy = hn.y * ui.x, vx = hn.x * ui.y, vy = hn.y * ui.y;
  int nb = 0;
  for (int k = 0; k < n; ++k) {
    const int64_t e = sell_entry(a.slice_e0, p, k);
    const int j = a.col[e];
    const double2 c = a.nxy[e];
    const double2 u = a.UV[j];
    ux = fma(c.x, u.x, ux); uy = fma(c.y, u.x, uy);
    vx = fma(c.x, u.y, vx); vy = fma(c.y, u.y, vy);
    if (corner || a.slice_g[j / kSlice] != 5) ++nb;
  }
  const double t = uy + vx;
  const double eps2 = (((ux * ux + vy * vy) + ux * vy) + 0.25 * (t * t)) + 1e-12;
  const double K1 = 2.0 * ux + vy, K2 = 0.5 * t, K3 = 2.0 * vy + ux;
  a.K[p] = K1; a.K[a.nP + p] = K2; a.K[2 * a.nP + p] = K3;
  a.inv_nb[p] = edge && nb > 0 ? 1.0 / (double)nb : 0.0;
  if (edge) {
    a.ee[p] = make_double2(1.0, 1.0); a.kh[p] = make_double2(0.0, 0.0); a.alpha[p] = make_double2(0.0, 0.0);
    a.dinv[p] = make_double2(1.0, 1.0); a.c3[p] = 0.0; a.eta[p] = 1.0; a.fr[p] = 0.0;
    return;
  }
  const double pexp = (1.0 - 3.0) / (2.0 * 3.0);
  const double eta = pow((a.m_enh * 0.5) * a.Af[p], -1.0 / 3.0) * pow(eps2, pexp);
  const double mH = fmax(0.1, a.Hi[p]);
  const bool floating = is_floating(a.Hi[p], a.Hb[p], a.SL[p]);
  // sliding coefficient at the converged velocities (SSA_sliding_term, ice_dynamics_module.f90:727-779)
  const double wv = (1e-3 * 1e-3 + ui.x * ui.x) + ui.y * ui.y;
  const double S = a.coulomb ? (a.tau[p] * pow(wv, a.expo)) / a.uq : (a.beta ? a.beta[p] : a.beta_const);
  const double fr = floating ? 0.0 : S / (mH * eta);
  const double rg = kIceDensity * kGrav;
  const double2 hc = a.h_cuv[p];
  // The Coulomb law's S depends on the row's own velocity: d(fr u)/du adds the symmetric 2x2
  // block 2 expo fr / w [U U, U V; V U, V V] (w = dv^2 + U^2 + V^2) to the row's diagonal and
  // cross coefficients.
  const double cS = (a.coulomb && !floating) ? (2.0 * a.expo) * fr / wv : 0.0;
  const double eu = hc.x - fr - cS * ui.x * ui.x, ev = hc.y - fr - cS * ui.y * ui.y;
  // dF/deta * deta/d(eps2): alpha = p (fr u + rho g h / eta) / eps2
  const double ax = pexp * (fr * ui.x + rg * a.hx[p] / eta) / eps2;
  const double ay = pexp * (fr * ui.y + rg * a.hy[p] / eta) / eps2;
  const double kU = K1 * hn.x + K2 * hn.y, kV = K2 * hn.x + K3 * hn.y;
  a.ee[p] = make_double2(eu, ev);
  a.c3[p] = 3.0 * a.sNxy[p] - cS * ui.x * ui.y;
  a.kh[p] = make_double2(kU, kV);
  a.alpha[p] = make_double2(ax, ay);
  a.dinv[p] = make_double2(1.0 / (eu + kU * ax), 1.0 / (ev + kV * ay));
  a.eta[p] = eta;
  a.fr[p] = fr;
}

// Transposed coefficients per entry: entry (p -> q) holds the coefficient of u_p in
// equation q, found through q's own entry (q -> p).
__global__ void k_adj_entries(const AdjSetup a, double2 *cT, double2 *kT, const double2 *cuv, AdjCtl *ctl) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.nP) return;
  const int n = a.deg[p];
  const bool p_edge = a.slice_g[p / kSlice] == 5;
  for (int k = 0; k < n; ++k) {
    const int64_t e = sell_entry(a.slice_e0, p, k);
    const int q = a.col[e];
    const int nq = a.deg[q];
    int64_t f = -1;
    for (int kk = 0; kk < nq; ++kk) {
      const int64_t e2 = sell_entry(a.slice_e0, q, kk);
      if (a.col[e2] == p) { f = e2; break; }
    }
    double2 c = make_double2(0.0, 0.0), kc = make_double2(0.0, 0.0);
    if (f < 0) {
      atomicAdd(&ctl->not_found, 1);
    } else if (a.slice_g[q / kSlice] == 5) {
      // q is an edge row (averages its non-edge neighbours) or a corner (all neighbours)
      const bool member = a.orig_of_dev[q] < 4 || !p_edge;
      if (member) c = make_double2(-a.inv_nb[q], -a.inv_nb[q]);
    } else {
      c = cuv[f];
      const double2 nq2 = a.nxy[f];
      const double K1 = a.K[q], K2 = a.K[a.nP + q], K3 = a.K[2 * a.nP + q];
      kc = make_double2(K1 * nq2.x + K2 * nq2.y, K2 * nq2.x + K3 * nq2.y);
    }
    cT[e] = c;
    kT[e] = kc;
  }
}

// Gradients per row (caller order out): dJ/dlog(beta^2), and the sensitivities to the
// gathered fields hx, hy and Hi_AaAc; the adjoint state itself.
struct AdjGrad {
  int nP, nV;
  const int *orig_of_dev;
  const uint8_t *deg;
  const uint8_t *slice_g;
  const double2 *UV, *mu;
  const double *eta, *fr, *Hi;
  int coulomb;
  const double *phi;                                       // Coulomb: till friction angle (degrees)
  double *d_logbeta, *s_hx, *s_hy, *s_H, *lam_U, *lam_V;   // [nA] caller order
  double *d_phi;                                           // [nA] caller order, Coulomb only
};

__global__ void k_adj_grad(const AdjGrad a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.nP) return;
  const int r = a.orig_of_dev[p];
  if (r < 0 || a.deg[p] == 0) return;
  const double2 m = a.mu[p];
  a.lam_U[r] = m.x;
  a.lam_V[r] = m.y;
  if (a.slice_g[p / kSlice] == 5) {
    a.d_logbeta[r] = 0.0; a.s_hx[r] = 0.0; a.s_hy[r] = 0.0; a.s_H[r] = 0.0;
    if (a.coulomb) a.d_phi[r] = 0.0;
    return;
  }
  const double2 u = a.UV[p];
  // S is proportional to beta^2 (linear law) or to tau_c (Coulomb law): dF/dlog(coefficient)
  // = -fr u on the row, so both laws share the gradient with respect to the log coefficient.
  const double w = a.fr[p] * fma(m.x, u.x, m.y * u.y);
  const double rg = kIceDensity * kGrav;
  a.d_logbeta[r] = w;
  a.s_hx[r] = rg * m.x / a.eta[p];
  a.s_hy[r] = rg * m.y / a.eta[p];
  // Coulomb: tau_c and the friction denominator both carry max(0.1, Hi), so the friction
  // term does not depend on the thickness.
  a.s_H[r] = (!a.coulomb && a.Hi[p] > 0.1) ? -w / a.Hi[p] : 0.0;
  if (a.coulomb) {
    // tau_c = tan(phi pi / 180) X (basal_yield_stress, 780-844): dlog(tau_c)/dphi = (pi / 180) / (sin cos)
    const double ph = a.phi[p] * (kPi / 180.0);
    a.d_phi[r] = w * (kPi / 180.0) / (sin(ph) * cos(ph));
  }
}

// dJ/dHi on Aa from the field sensitivities: Hi_AaAc (identity on Aa rows, the mean of the
// two end vertices on Ac rows) and the driving-stress slopes (Aa and Ac derivative
// stencils of Hs, or (1 - rho_i/rho_sw) times those of Hi on floating rows), masks frozen.
struct AdjGeom {
  int nV, nAc, ncm;
  const int *dev_of_orig;
  const double *Hi, *Hb, *SL;        // device order fields
  const double *s_hx, *s_hy, *s_H;   // caller order sensitivities
  const int *nC, *C;                 // (nV), (nV, ncm) 1-based
  const double *Nx, *Ny;             // (nV, ncm + 1)
  const int *Aci;                    // (nAc, 4) 1-based
  const double *Nx_Ac, *Ny_Ac;       // (nAc, 4)
  double *dHi;                       // (nV), zeroed
};

__device__ __forceinline__ double hs_slope(const AdjGeom &a, int v) {
  const int p = a.dev_of_orig[v];
  return is_floating(a.Hi[p], a.Hb[p], a.SL[p]) ? 1.0 - kIceDensity / kSeawaterDensity : 1.0;
}

__global__ void k_adj_geom(const AdjGeom a) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int nA = a.nV + a.nAc;
  if (r >= nA) return;
  const double shx = a.s_hx[r], shy = a.s_hy[r], sH = a.s_H[r];
  const int p = a.dev_of_orig[r];
  const bool ocean = is_floating(a.Hi[p], a.Hb[p], a.SL[p]);
  const double shelf = 1.0 - kIceDensity / kSeawaterDensity;
  if (r < a.nV) {
    const int v = r;
    if (sH != 0.0) atomicAdd(&a.dHi[v], sH);
    if (shx == 0.0 && shy == 0.0) return;
    const int n = a.nC[v];
    for (int c = 0; c <= n; ++c) {
      const int k = c < n ? a.C[v + (size_t)c * a.nV] - 1 : v;
      const double fac = ocean ? shelf : hs_slope(a, k);
      const double w = shx * a.Nx[v + (size_t)c * a.nV] + shy * a.Ny[v + (size_t)c * a.nV];
      atomicAdd(&a.dHi[k], w * fac);
    }
  } else {
    const int ac = r - a.nV;
    if (sH != 0.0) {
      atomicAdd(&a.dHi[a.Aci[ac] - 1], 0.5 * sH);
      atomicAdd(&a.dHi[a.Aci[ac + a.nAc] - 1], 0.5 * sH);
    }
    if (shx == 0.0 && shy == 0.0) return;
    for (int c = 0; c < 4; ++c) {
      const int k = a.Aci[ac + (size_t)c * a.nAc] - 1;
      if (k < 0) continue;
      const double fac = ocean ? shelf : hs_slope(a, k);
      const double w = shx * a.Nx_Ac[ac + (size_t)c * a.nAc] + shy * a.Ny_Ac[ac + (size_t)c * a.nAc];
      atomicAdd(&a.dHi[k], w * fac);
    }
  }
}

// ---------------------------------------------------------------------------------------
// Gather / scatter / GL flux
// ---------------------------------------------------------------------------------------
struct StageIn {   // device staging of the caller's arrays (original order)
  const double *Hi, *Hb, *SL, *hx, *hy, *Af;          // Aa (nV)
  const double *Hi_Ac, *Hb_Ac, *SL_Ac, *hx_Ac, *hy_Ac, *Af_Ac;  // Ac (nAc)
  const double *beta;                                  // (nA) or null
  const double *U, *V, *Ux, *Uy;                       // warm start
  const double *N;                                     // (nA) or null
};

struct Fields {
  double *Hi, *Hb, *SL, *hx, *hy, *Af, *beta, *tau, *phi;
  double2 *UV;
  float2 *dUV;
  double *Na, *Nb;
};

// Gather into device order, and basal_yield_stress (Martin et al. 2011) per row.
__global__ void k_gather(int nP, int nV, const int *orig_of_dev, StageIn in, Fields f) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nP) return;
  const int r = orig_of_dev[p];
  if (r < 0) {
    f.Hi[p] = 0.0; f.Hb[p] = 0.0; f.SL[p] = 0.0; f.hx[p] = 0.0; f.hy[p] = 0.0; f.Af[p] = 1.0;
    f.tau[p] = 0.0; f.phi[p] = 0.0; f.UV[p] = make_double2(0.0, 0.0); f.dUV[p] = make_float2(0.f, 0.f);
    f.Na[p] = 0.0; f.Nb[p] = 0.0;
    if (f.beta) f.beta[p] = 0.0;
    return;
  }
  double Hi, Hb, SL, hx, hy, Af, U, V;
  if (r < nV) {
    Hi = in.Hi[r]; Hb = in.Hb[r]; SL = in.SL[r]; hx = in.hx[r]; hy = in.hy[r]; Af = in.Af[r];
    U = in.U[r]; V = in.V[r];
  } else {
    const int a = r - nV;
    Hi = in.Hi_Ac[a]; Hb = in.Hb_Ac[a]; SL = in.SL_Ac[a]; hx = in.hx_Ac[a]; hy = in.hy_Ac[a]; Af = in.Af_Ac[a];
    U = in.Ux[a]; V = in.Uy[a];
  }
  f.Hi[p] = Hi; f.Hb[p] = Hb; f.SL[p] = SL; f.hx[p] = hx; f.hy[p] = hy; f.Af[p] = Af;
  f.UV[p] = make_double2(U, V);
  f.dUV[p] = make_float2(0.f, 0.f);
  const double Nin = in.N ? in.N[r] : 0.0;
  f.Na[p] = Nin;
  f.Nb[p] = Nin;
  if (f.beta) f.beta[p] = in.beta ? in.beta[r] : 0.0;
  // basal_yield_stress, ice_dynamics_module.f90:780-844
  const double pf1 = -1000.0, pf2 = 0.0, p_min = 5.0, p_max = 20.0;
  const double lambda_p = fmax(0.0, fmin(1.0, (1.0 - (Hb - SL) / 1000.0)));
  const double pwp = (((0.96 * kIceDensity) * kGrav) * fmax(0.1, Hi)) * lambda_p;
  const double phi = fmax(p_min, fmin(p_max, (p_min + (p_max - p_min) * (1.0 + (Hb - pf2) / (pf2 - pf1)))));
  f.phi[p] = phi;
  f.tau[p] = tan((kPi / 180.0) * phi) * (((kIceDensity * kGrav) * fmax(0.1, Hi)) - pwp);
}

struct GlIn {
  const int *mask_gl_Ac, *mask_sheet;
  const double *Hi, *Hb, *SL, *Af;   // Aa
  const double *dHi_dx, *dHi_dy, *dSL_dx, *dSL_dy, *dHb_dx, *dHb_dy;  // Ac
};

__device__ double norm2_scaled(double a, double b) {
  // NORM2([a,b]) as gfortran evaluates it: scaled one-pass sum of squares.
  double scale = 0.0, ssq = 1.0;
  const double v[2] = {a, b};
  for (int i = 0; i < 2; ++i) {
    if (v[i] != 0.0) {
      const double ax = fabs(v[i]);
      if (scale < ax) {
        const double r = scale / ax;
        ssq = 1.0 + (ssq * r) * r;
        scale = ax;
      } else {
        const double r = ax / scale;
        ssq = ssq + r * r;
      }
    }
  }
  return scale * sqrt(ssq);
}

// calculate_GL_flux (Tsai et al. 2015 flux for the Coulomb law), ice_dynamics_module.f90:848-949:
// prescribes Ux/Uy on grounding-line Ac rows and marks them as skipped by the sweep.
__global__ void k_gl_flux(int nAc, int nV, const int *dev_of_orig, const int2 *Aci12, GlIn g,
                          const double *phi_dev, double2 *UV, uint8_t *skip, double factor_const) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nAc) return;
  const int p = dev_of_orig[nV + a];
  skip[p] = 0;
  if (g.mask_gl_Ac[a] == 0) return;
  const int vi = Aci12[a].x, vj = Aci12[a].y;
  const double rsw = kSeawaterDensity / kIceDensity;
  const double TAFi = g.Hi[vi] - ((g.SL[vi] - g.Hb[vi]) * rsw);
  const double TAFj = g.Hi[vj] - ((g.SL[vj] - g.Hb[vj]) * rsw);
  const double lambda_GL = TAFi / (TAFi - TAFj);
  const double Hi_GL = (g.Hi[vi] * (1.0 - lambda_GL)) + (g.Hi[vj] * lambda_GL);
  double phi_GL, A_GL;
  if (g.mask_sheet[vi] == 1) { phi_GL = phi_dev[dev_of_orig[vi]]; A_GL = g.Af[vi]; }
  else { phi_GL = phi_dev[dev_of_orig[vj]]; A_GL = g.Af[vj]; }
  // factor_const = (8 Q0) then * A * (rho g)^n * (1 - rho_i/rho_sw)^(n-1) / 4^n, n = 3
  const double one_m = 1.0 - (kIceDensity / kSeawaterDensity);
  const double factor_Tsai = (((factor_const * A_GL) * pow(kIceDensity * kGrav, 3.0)) * (one_m * one_m)) / pow(4.0, 3.0);
  const double Qabs = (factor_Tsai * pow(Hi_GL, 3.0 + 2.0)) / tan(phi_GL * (kPi / 180.0));
  double Fx = -(g.dHi_dx[a] - ((g.dSL_dx[a] - g.dHb_dx[a]) * rsw));
  double Fy = -(g.dHi_dy[a] - ((g.dSL_dy[a] - g.dHb_dy[a]) * rsw));
  const double F = norm2_scaled(Fx, Fy);
  Fx = Fx / F;
  Fy = Fy / F;
  UV[p] = make_double2((Qabs * Fx) / Hi_GL, (Qabs * Fy) / Hi_GL);
  skip[p] = 1;
}

struct StageOut {
  double *U, *V, *Ux, *Uy, *Up, *Uo;   // Aa (nV) / Ac (nAc)
  double *N, *eta, *S, *tau, *phi;     // (nA)
};

__global__ void k_scatter(int nA, int nV, const int *dev_of_orig, const double2 *V, const int2 *Aci12,
                          const double2 *UV, const double *N, const double *eta, const double *S,
                          const double *tau, const double *phi, StageOut o) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nA) return;
  const int p = dev_of_orig[r];
  const double2 u = UV[p];
  o.N[r] = N[p];
  o.eta[r] = eta[p];
  o.S[r] = S[p];
  o.tau[r] = tau[p];
  o.phi[r] = phi[p];
  if (r < nV) {
    o.U[r] = u.x;
    o.V[r] = u.y;
  } else {
    const int a = r - nV;
    o.Ux[a] = u.x;
    o.Uy[a] = u.y;
    const int2 ij = Aci12[a];
    const double Dx = V[ij.y].x - V[ij.x].x;
    const double Dy = V[ij.y].y - V[ij.x].y;
    const double D = sqrt(Dx * Dx + Dy * Dy);
    o.Up[a] = (u.x * Dx) / D + (u.y * Dy) / D;
    o.Uo[a] = (u.y * Dx) / D - (u.x * Dy) / D;
  }
}

// ---------------------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------------------

// Limit of every device-side bounded wait (team barriers, neighbour progress waits, lagged
// decisions): 20 s, or the positive integer in UFE_WAIT_TIMEOUT_NS. The tests set a few
// nanoseconds to make the waits run out and check that the solve reports UFE_TIMEOUT and the
// context stays usable; nothing else should set it.
long long wait_timeout_ns() {
  const char *env = std::getenv("UFE_WAIT_TIMEOUT_NS");
  if (env && *env) {
    const long long v = std::atoll(env);
    if (v > 0) return v;
  }
  return 20LL * 1000 * 1000 * 1000;
}
struct SsaWork {
  int nP = 0, nV = 0, nAc = 0, nA = 0;
  // staging (original order)
  double *stage_in = nullptr;    // 12 nV-or-nAc fields + beta + warm start + N
  double *stage_out = nullptr;
  int *gl_int = nullptr;         // mask_gl_Ac (nAc) + mask_sheet (nV)
  double *gl_dbl = nullptr;      // 6 Ac slope fields
  // device-order fields
  double *f = nullptr;           // Hi, Hb, SL, hx, hy, Af, beta, tau, phi, eta, Na, Nb, S
  double2 *UV = nullptr, *rhs = nullptr, *euv = nullptr, *rcp = nullptr;
  float2 *dUV = nullptr, *r0 = nullptr, *rcp32 = nullptr;
  double2 *UVb = nullptr, *UVc = nullptr;   // halo sweeps: second and third velocity buffers (FP64 modes)
  float2 *dUVb = nullptr, *dUVc = nullptr;  // halo sweeps: second and third correction buffers (mixed)
  float4 *hsd32 = nullptr;       // halo sweeps: per-slot row data (mixed)
  double2 *hrcp = nullptr, *hrhs = nullptr;   // halo sweeps: per-slot row data (fast FP64)
  float4 *bc0 = nullptr;         // mixed: boundary offsets per edge ordinal
  uint8_t *skip = nullptr;
  double *rn_part = nullptr;
  unsigned int *prog = nullptr;
  double *fh = nullptr;          // frictional heating out (nV) + mask (nV ints), on first use
  SsaCtl *ctl = nullptr;
  SsaCtl *ctl_host = nullptr;    // pinned
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // state of the last upload
  bool uploaded = false;
  bool has_beta = false, has_N = false, gl = false;
  bool zero = false;             // the reference's early-out applies
  int sliding_law = -1;          // law of the last prepared solve
  bool halo_used = false;        // the last single solve ran the halo sweeps
  int grid[3] = {0, 0, 0};        // per SweepMode, one CTA per SM
  int block = kSsaBlock;
};

void ssa_free(SsaWork *w) {
  if (!w) return;
  void *ptrs[] = {w->stage_in, w->stage_out, w->gl_int, w->gl_dbl, w->f, w->UV, w->rhs, w->euv,
                  w->rcp, w->dUV, w->r0, w->rcp32, w->skip, w->rn_part, w->prog, w->ctl, w->fh,
                  w->UVb, w->dUVb, w->UVc, w->dUVc, w->hsd32, w->hrcp, w->hrhs, w->bc0};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (w->ctl_host) cudaFreeHost(w->ctl_host);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

namespace {

enum { F_HI, F_HB, F_SL, F_HX, F_HY, F_AF, F_BETA, F_TAU, F_PHI, F_ETA, F_NA, F_NB, F_S, F_COUNT };
// stage_in layout (doubles): Aa block 6*nV, Ac block 6*nAc, beta nA, U nV, V nV, Ux nAc, Uy nAc, N nA
// stage_out layout: U nV, V nV, Ux nAc, Uy nAc, Up nAc, Uo nAc, N nA, eta nA, S nA, tau nA, phi nA

int ensure_work(ufe_mesh_h h) {
  if (h->ssa) return UFE_OK;
  const DevMesh &m = h->m;
  SsaWork *w = new SsaWork();
  w->nP = m.nP; w->nV = m.nV; w->nAc = m.nAc; w->nA = m.nA;
  const size_t nin = 6 * (size_t)m.nV + 6 * (size_t)m.nAc + 2 * (size_t)m.nA + 2 * (size_t)m.nV + 2 * (size_t)m.nAc;
  const size_t nout = 2 * (size_t)m.nV + 4 * (size_t)m.nAc + 5 * (size_t)m.nA;
  int rc = cuda_status(cudaMalloc(&w->stage_in, nin * sizeof(double)), "ssa stage_in");
  if (!rc) rc = cuda_status(cudaMalloc(&w->stage_out, nout * sizeof(double)), "ssa stage_out");
  if (!rc) rc = cuda_status(cudaMalloc(&w->gl_int, ((size_t)m.nAc + m.nV) * sizeof(int)), "ssa gl_int");
  if (!rc) rc = cuda_status(cudaMalloc(&w->gl_dbl, 6 * (size_t)m.nAc * sizeof(double)), "ssa gl_dbl");
  if (!rc) rc = cuda_status(cudaMalloc(&w->f, (size_t)F_COUNT * m.nP * sizeof(double)), "ssa fields");
  if (!rc) rc = cuda_status(cudaMalloc(&w->UV, (size_t)m.nP * sizeof(double2)), "ssa UV");
  if (!rc) rc = cuda_status(cudaMalloc(&w->rhs, (size_t)m.nP * sizeof(double2)), "ssa rhs");
  if (!rc) rc = cuda_status(cudaMalloc(&w->euv, (size_t)m.nP * sizeof(double2)), "ssa euv");
  if (!rc) rc = cuda_status(cudaMalloc(&w->dUV, (size_t)m.nP * sizeof(float2)), "ssa dUV");
  if (!rc) rc = cuda_status(cudaMalloc(&w->r0, (size_t)m.nP * sizeof(float2)), "ssa r0");
  if (!rc) rc = cuda_status(cudaMalloc(&w->rcp, (size_t)m.nP * sizeof(double2)), "ssa rcp");
  if (!rc) rc = cuda_status(cudaMalloc(&w->rcp32, (size_t)m.nP * sizeof(float2)), "ssa rcp32");
  if (!rc) rc = cuda_status(cudaMalloc(&w->skip, (size_t)m.nP), "ssa skip");
  if (!rc) rc = cuda_status(cudaMalloc(&w->bc0, ((size_t)m.n_edge_total + 1) * sizeof(float4)), "ssa bc0");
  if (!rc && m.has_halo) rc = cuda_status(cudaMalloc(&w->UVb, (size_t)m.nP * sizeof(double2)), "ssa UVb");
  if (!rc && m.has_halo) rc = cuda_status(cudaMalloc(&w->dUVb, (size_t)m.nP * sizeof(float2)), "ssa dUVb");
  if (!rc && m.has_halo) rc = cuda_status(cudaMalloc(&w->UVc, (size_t)m.nP * sizeof(double2)), "ssa UVc");
  if (!rc && m.has_halo) rc = cuda_status(cudaMalloc(&w->dUVc, (size_t)m.nP * sizeof(float2)), "ssa dUVc");
  const size_t nslots = (size_t)m.n_hslices * kSlice;
  if (!rc && m.has_halo) rc = cuda_status(cudaMalloc(&w->hsd32, nslots * sizeof(float4)), "ssa hsd32");
  if (!rc && m.has_halo) rc = cuda_status(cudaMalloc(&w->hrcp, nslots * sizeof(double2)), "ssa hrcp");
  if (!rc && m.has_halo) rc = cuda_status(cudaMalloc(&w->hrhs, nslots * sizeof(double2)), "ssa hrhs");
  if (!rc) rc = cuda_status(cudaMalloc(&w->ctl, sizeof(SsaCtl)), "ssa ctl");
  if (!rc) rc = cuda_status(cudaMallocHost(&w->ctl_host, sizeof(SsaCtl)), "ssa ctl host");
  if (!rc) rc = cuda_status(cudaEventCreate(&w->ev0), "event");
  if (!rc) rc = cuda_status(cudaEventCreate(&w->ev1), "event");
  if (!rc) rc = cuda_status(cudaMemsetAsync(w->skip, 0, (size_t)m.nP, h->stream), "memset skip");
  // Persistent grid: every CTA co-resident (cooperative launch), one CTA of 1024 threads per SM.
  const void *kernels[5] = {(const void *)ssa_persistent<kExact64, false>, (const void *)ssa_persistent<kFast64, false>,
                            (const void *)ssa_persistent<kMixed, false>, (const void *)ssa_persistent<kFast64, true>,
                            (const void *)ssa_persistent<kMixed, true>};
  int gmax = 0;
  for (int k = 0; k < 5 && !rc; ++k) {
    if (k >= 3 && !m.has_halo) break;
    int per_sm = 0;
    rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernels[k], k >= 3 ? kHaloBlock : w->block, 0),
                     "occupancy");
    if (!rc && per_sm * h->num_sms < m.n_patch) {
      set_error("ssa kernel: not enough co-resident CTAs for one per patch");
      rc = UFE_CUDA_ERROR;
    }
    if (k < 3) w->grid[k] = m.n_patch;   // one CTA per patch (n_patch <= kCtasPerSm * number of SMs)
    gmax = gmax > m.n_patch ? gmax : m.n_patch;
  }
  if (!rc) rc = cuda_status(cudaMalloc(&w->rn_part, 2 * (size_t)gmax * sizeof(double)), "rn_part");
  if (!rc) rc = cuda_status(cudaMalloc(&w->prog, 32 * (size_t)gmax * sizeof(unsigned int)), "progress counters");
  if (rc) { ssa_free(w); return rc; }
  h->ssa = w;
  return UFE_OK;
}

int h2d(double *dst, const double *src, size_t n, cudaStream_t s) {
  return cuda_status(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, s), "H2D");
}
int d2h(double *dst, const double *src, size_t n, cudaStream_t s) {
  if (!dst) return UFE_OK;
  return cuda_status(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H");
}

}  // namespace

}  // namespace ufe

using namespace ufe;

namespace ufe {
// ufe_ssa_upload; with in_on_device the arrays of `in` are device arrays of this device (the
// device geometry preparation) and sheet_count is the number of grounded-ice vertices.
int ssa_upload_impl(ufe_mesh_h h, const ufe_params *p, const ufe_ssa_in *in, const ufe_ssa_inout *io,
                    bool in_on_device, long long sheet_count) {
  if (!h || !p || !in || !io) { set_error(std::string(in_on_device ? "ufe_ssa_upload_geometry" : "ufe_ssa_upload") + ": null argument"); return UFE_BAD_ARG; }
  if (!in->Hi || !in->Hb || !in->SL || !in->dHs_dx_shelf || !in->dHs_dy_shelf || !in->A_flow_mean ||
      !in->mask_sheet || !in->Hi_Ac || !in->Hb_Ac || !in->SL_Ac || !in->dHs_dx_shelf_Ac ||
      !in->dHs_dy_shelf_Ac || !in->A_flow_mean_Ac || !io->U_SSA || !io->V_SSA || !io->Ux_SSA_Ac || !io->Uy_SSA_Ac) {
    set_error(std::string(in_on_device ? "ufe_ssa_upload_geometry" : "ufe_ssa_upload") + ": missing input array");
    return UFE_BAD_ARG;
  }
  if (p->use_analytical_GL_flux && (!in->mask_gl_Ac || !in->dHi_dx_Ac || !in->dHi_dy_Ac || !in->dSL_dx_Ac ||
                                    !in->dSL_dy_Ac || !in->dHb_dx_Ac || !in->dHb_dy_Ac)) {
    set_error(std::string(in_on_device ? "ufe_ssa_upload_geometry" : "ufe_ssa_upload") + ": use_analytical_GL_flux needs mask_gl_Ac and the Ac slopes of Hi, SL, Hb");
    return UFE_BAD_ARG;
  }
  if (p->use_analytical_GL_flux && p->sliding_law != UFE_SLIDING_COULOMB_REGULARISED) {
    set_error(std::string(in_on_device ? "ufe_ssa_upload_geometry" : "ufe_ssa_upload") + ": the GL flux is implemented for the Coulomb_regularised law only (as in the reference)");
    return UFE_BAD_ARG;
  }
  int rc = ensure_work(h);
  if (rc) return rc;
  SsaWork *w = h->ssa;
  const size_t nV = w->nV, nAc = w->nAc, nA = w->nA;
  cudaStream_t s = h->stream;
  double *st = w->stage_in;
  const double *aa[6] = {in->Hi, in->Hb, in->SL, in->dHs_dx_shelf, in->dHs_dy_shelf, in->A_flow_mean};
  const double *ac[6] = {in->Hi_Ac, in->Hb_Ac, in->SL_Ac, in->dHs_dx_shelf_Ac, in->dHs_dy_shelf_Ac, in->A_flow_mean_Ac};
  const cudaMemcpyKind kin = in_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  auto cp = [&](double *dst, const double *src, size_t n) {
    return cuda_status(cudaMemcpyAsync(dst, src, n * sizeof(double), kin, s), "upload");
  };
  for (int k = 0; k < 6 && !rc; ++k) rc = cp(st + k * nV, aa[k], nV);
  for (int k = 0; k < 6 && !rc; ++k) rc = cp(st + 6 * nV + k * nAc, ac[k], nAc);
  double *beta = st + 6 * nV + 6 * nAc;
  double *U = beta + nA, *V = U + nV, *Ux = V + nV, *Uy = Ux + nAc, *N = Uy + nAc;
  w->has_beta = in->beta_sq_AaAc != nullptr;
  if (!rc && w->has_beta) rc = cp(beta, in->beta_sq_AaAc, nA);
  if (!rc) rc = h2d(U, io->U_SSA, nV, s);
  if (!rc) rc = h2d(V, io->V_SSA, nV, s);
  if (!rc) rc = h2d(Ux, io->Ux_SSA_Ac, nAc, s);
  if (!rc) rc = h2d(Uy, io->Uy_SSA_Ac, nAc, s);
  w->has_N = io->N_AaAc != nullptr;
  if (!rc && w->has_N) rc = h2d(N, io->N_AaAc, nA, s);
  w->gl = p->use_analytical_GL_flux != 0;
  if (!rc && w->gl) {
    rc = cuda_status(cudaMemcpyAsync(w->gl_int, in->mask_gl_Ac, nAc * sizeof(int), kin, s), "upload");
    if (!rc) rc = cuda_status(cudaMemcpyAsync(w->gl_int + nAc, in->mask_sheet, nV * sizeof(int), kin, s), "upload");
    const double *gs[6] = {in->dHi_dx_Ac, in->dHi_dy_Ac, in->dSL_dx_Ac, in->dSL_dy_Ac, in->dHb_dx_Ac, in->dHb_dy_Ac};
    for (int k = 0; k < 6 && !rc; ++k) rc = cp(w->gl_dbl + k * nAc, gs[k], nAc);
  }
  // Early-outs of solve_SSA (431-452): benchmark experiments without SSA, or no grounded ice.
  long long sheet = sheet_count;
  if (!in_on_device)
    for (size_t v = 0; v < nV; ++v) sheet += in->mask_sheet[v];
  w->zero = p->zero_velocities != 0 || sheet == 0;
  w->uploaded = rc == UFE_OK;
  return rc;
}
}  // namespace ufe

namespace ufe {
// U_SSA then V_SSA (nV each) of the last solve on this handle, on the device, or null.
const double *ssa_device_UV(ufe_mesh_h h) {
  const SsaWork *w = h->ssa;
  if (!w || !w->uploaded) return nullptr;
  return w->stage_out;
}
// Up_SSA_Ac of the last solve on this handle, on the device (caller order), or null.
const double *ssa_device_Up(ufe_mesh_h h) {
  const SsaWork *w = h->ssa;
  if (!w || !w->uploaded) return nullptr;
  return w->stage_out + 2 * (size_t)w->nV + 2 * (size_t)w->nAc;
}
}  // namespace ufe

extern "C" int ufe_ssa_upload(ufe_mesh_h h, const ufe_params *p, const ufe_ssa_in *in, const ufe_ssa_inout *io) {
  return ssa_upload_impl(h, p, in, io, false, 0);
}

namespace ufe {
namespace {

int check_params(const ufe_params *p, const char *who) {
  if (p->precision != UFE_FP64 && p->precision != UFE_MIXED) { set_error(std::string(who) + ": unknown precision"); return UFE_BAD_ARG; }
  if (p->sliding_law != UFE_SLIDING_COULOMB_REGULARISED && p->sliding_law != UFE_SLIDING_LINEAR) {
    set_error(std::string(who) + ": sliding law not implemented");
    return UFE_BAD_ARG;
  }
  if (p->SSA_max_inner_loops < 1 || p->SSA_max_outer_loops < 1) {
    set_error(std::string(who) + ": loop limits must be >= 1");
    return UFE_BAD_ARG;
  }
  return UFE_OK;
}

int sweep_mode(const ufe_params *p) {
  return p->precision == UFE_MIXED ? kMixed : (p->fp64_exact ? kExact64 : kFast64);
}

Fields fields_of(SsaWork *w) {
  const size_t nP = w->nP;
  double *F = w->f;
  Fields fl;
  fl.Hi = F + F_HI * nP; fl.Hb = F + F_HB * nP; fl.SL = F + F_SL * nP; fl.hx = F + F_HX * nP;
  fl.hy = F + F_HY * nP; fl.Af = F + F_AF * nP; fl.beta = w->has_beta ? F + F_BETA * nP : nullptr;
  fl.tau = F + F_TAU * nP; fl.phi = F + F_PHI * nP; fl.UV = w->UV; fl.dUV = w->dUV;
  fl.Na = F + F_NA * nP; fl.Nb = F + F_NB * nP;
  return fl;
}

// Gather the uploaded inputs into device order (and the GL flux rows), clear the control
// block, and fill the argument block of the persistent solver. Returns *solve = false when
// the reference's early-out applies (no solve to run).
int launch_prepare(ufe_mesh_h h, const ufe_params *p, cudaStream_t s, SsaArgs *a, bool *solve) {
  SsaWork *w = h->ssa;
  const DevMesh &m = h->m;
  const size_t nV = w->nV, nAc = w->nAc, nA = w->nA, nP = w->nP;
  Fields fl = fields_of(w);
  double *F = w->f;
  double *st = w->stage_in;
  StageIn si;
  si.Hi = st; si.Hb = st + nV; si.SL = st + 2 * nV; si.hx = st + 3 * nV; si.hy = st + 4 * nV; si.Af = st + 5 * nV;
  double *acb = st + 6 * nV;
  si.Hi_Ac = acb; si.Hb_Ac = acb + nAc; si.SL_Ac = acb + 2 * nAc; si.hx_Ac = acb + 3 * nAc;
  si.hy_Ac = acb + 4 * nAc; si.Af_Ac = acb + 5 * nAc;
  si.beta = w->has_beta ? acb + 6 * nAc : nullptr;
  si.U = acb + 6 * nAc + nA; si.V = si.U + nV; si.Ux = si.V + nV; si.Uy = si.Ux + nAc;
  si.N = w->has_N ? si.Uy + nAc : nullptr;
  int rc = cuda_status(cudaMemsetAsync(w->ctl, 0, sizeof(SsaCtl), s), "memset ctl");
  if (!rc) {
    k_gather<<<(unsigned)((nP + 255) / 256), 256, 0, s>>>((int)nP, (int)nV, m.orig_of_dev, si, fl);
    rc = cuda_status(cudaGetLastError(), "k_gather");
  }
  if (!rc && w->gl && !w->zero) {
    GlIn g;
    g.mask_gl_Ac = w->gl_int; g.mask_sheet = w->gl_int + nAc;
    g.Hi = si.Hi; g.Hb = si.Hb; g.SL = si.SL; g.Af = si.Af;
    g.dHi_dx = w->gl_dbl; g.dHi_dy = w->gl_dbl + nAc; g.dSL_dx = w->gl_dbl + 2 * nAc;
    g.dSL_dy = w->gl_dbl + 3 * nAc; g.dHb_dx = w->gl_dbl + 4 * nAc; g.dHb_dy = w->gl_dbl + 5 * nAc;
    k_gl_flux<<<(unsigned)((nAc + 255) / 256), 256, 0, s>>>((int)nAc, (int)nV, m.dev_of_orig, m.Aci12, g, fl.phi, w->UV, w->skip, 8.0 * 0.61);
    rc = cuda_status(cudaGetLastError(), "k_gl_flux");
  }
  if (!rc) rc = cuda_status(cudaMemsetAsync(F + F_S * nP, 0, nP * sizeof(double), s), "memset S");
  if (!rc) rc = cuda_status(cudaMemsetAsync(w->prog, 0, 32 * (size_t)m.n_patch * sizeof(unsigned int), s), "memset prog");
  *solve = !w->zero;
  std::memset(a, 0, sizeof(*a));
  a->col = m.col; a->cuv = m.cuv; a->nxy = m.nxy; a->cuv32 = m.cuv32; a->nxy32 = m.nxy32; a->deg = m.deg;
  a->slice_ptr = m.slice_ptr; a->h_nxy = m.h_nxy; a->h_cuv = m.h_cuv; a->sNxy = m.sNxy;
  a->s3Nxy = m.s3Nxy; a->h_nxy32 = m.h_nxy32; a->s3Nxy32 = m.s3Nxy32; a->bnd_ptr = m.bnd_ptr; a->bnd_nbr = m.bnd_nbr;
  a->slice_e0 = m.slice_e0; a->slice_w = m.slice_w; a->slice_g = m.slice_g; a->patch_slice = m.patch_slice;
  a->patch_edge0 = m.patch_edge0; a->edge_row = m.edge_row; a->sync_ptr = m.sync_ptr; a->sync_list = m.sync_list;
  a->hp_slice = m.hp_slice; a->hslice_e0 = m.hslice_e0; a->hslice_w = m.hslice_w; a->hrow_l = m.hrow_l;
  a->hrow_g = m.hrow_g; a->hcol = m.hcol; a->hcuv32 = m.hcuv32; a->hcuv = m.hcuv; a->hload_ptr = m.hload_ptr;
  a->hload_dev = m.hload_dev; a->hsync_ptr = m.hsync_ptr; a->hsync_list = m.hsync_list;
  a->UVb = w->UVb; a->dUVb = w->dUVb; a->UVc = w->UVc; a->dUVc = w->dUVc; a->hs3_32 = m.hs3_32; a->hs3 = m.hs3;
  a->hp_split = m.hp_split;
  a->hsd32 = w->hsd32; a->hrcp = w->hrcp; a->hrhs = w->hrhs;
  a->bc0 = w->bc0; a->n_edge = m.n_edge_total;
  a->prog = w->prog; a->nP = m.nP; a->nSlices = m.nSlices; a->ncm = m.ncm;
  a->Hi = fl.Hi; a->Hb = fl.Hb; a->SL = fl.SL; a->hx = fl.hx; a->hy = fl.hy; a->Af = fl.Af;
  a->beta = fl.beta; a->tau = fl.tau;
  a->skip = w->gl ? w->skip : nullptr;
  a->UV = w->UV; a->dUV = w->dUV; a->r0 = w->r0; a->rcp32 = w->rcp32; a->rcp = w->rcp;
  a->eta = F + F_ETA * nP; a->Na = fl.Na; a->Nb = fl.Nb; a->S = F + F_S * nP;
  a->rhs = w->rhs; a->euv = w->euv; a->rn_part = w->rn_part; a->ctl = w->ctl;
  a->omega = p->SSA_SOR_omega; a->tol = p->SSA_max_residual_UV; a->rn_tol = p->SSA_RN_tol;
  a->m_enh = p->m_enh_ssa;
  a->uq = std::pow(100.0, 0.30);          // u_threshold**q_plastic
  a->expo = 0.5 * (0.30 - 1.0);           // 0.5*(q_plastic-1)
  a->beta_const = p->beta_sq;
  a->max_inner = p->SSA_max_inner_loops; a->max_outer = p->SSA_max_outer_loops;
  a->sliding_law = p->sliding_law; a->has_beta = w->has_beta;
  w->sliding_law = p->sliding_law;
  // 256 on the 200k dome: 221.7 ms per solve against 226.0 at 128 and 234.2 at 64 (halo sweeps
  // before the resident slices), with the same error against the FP64 solve (1.17e-7) and the
  // same sweep count within one
  a->refold = p->mixed_refold_sweeps > 0 ? p->mixed_refold_sweeps : 256;
  a->fp32_visc = p->mixed_fp32_viscosity != 0;
  a->timeout_ns = wait_timeout_ns();
  return rc;
}

// Scatter the results back to the caller's order and fetch the control block.
int launch_finish(ufe_mesh_h h, cudaStream_t s) {
  SsaWork *w = h->ssa;
  const DevMesh &m = h->m;
  const size_t nV = w->nV, nAc = w->nAc, nA = w->nA, nP = w->nP;
  Fields fl = fields_of(w);
  double *F = w->f;
  StageOut o;
  double *so = w->stage_out;
  o.U = so; o.V = so + nV; o.Ux = so + 2 * nV; o.Uy = o.Ux + nAc; o.Up = o.Uy + nAc; o.Uo = o.Up + nAc;
  o.N = o.Uo + nAc; o.eta = o.N + nA; o.S = o.eta + nA; o.tau = o.S + nA; o.phi = o.tau + nA;
  int rc = UFE_OK;
  if (w->zero) rc = cuda_status(cudaMemsetAsync(w->UV, 0, nP * sizeof(double2), s), "memset UV");
  if (!rc) {
    k_scatter<<<(unsigned)((nA + 255) / 256), 256, 0, s>>>((int)nA, (int)nV, m.dev_of_orig, m.V, m.Aci12, w->UV,
                                                          fl.Na, F + F_ETA * nP, F + F_S * nP, fl.tau, fl.phi, o);
    rc = cuda_status(cudaGetLastError(), "k_scatter");
  }
  if (!rc) rc = cuda_status(cudaMemcpyAsync(w->ctl_host, w->ctl, sizeof(SsaCtl), cudaMemcpyDeviceToHost, s), "ctl D2H");
  return rc;
}

int stats_of(const SsaCtl &c, ufe_ssa_stats *stats, double ms) {
  int status = UFE_OK;
  if (c.err) {
    status = c.err;
    set_error("solve_SSA: a device-side bounded wait timed out");
  } else if (c.status == UFE_DIVERGED) {
    status = UFE_DIVERGED;
    set_error("solve_SSA: SSA remains unstable after resetting velocities to zero");
  } else if (c.resets == 1) {
    status = UFE_RESET_ONCE;
  } else if (c.not_converged > 0) {
    status = UFE_NOT_CONVERGED;
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->status = status;
    stats->picard_iterations = c.picard_iterations;
    stats->linear_solves = c.linear_solves;
    stats->resets = c.resets;
    stats->not_converged = c.not_converged;
    stats->total_sweeps = c.total_sweeps;
    stats->last_RN = c.last_RN;
    stats->last_max_residual = c.last_max_residual;
    for (int k = 0; k < 64; ++k) stats->sweeps[k] = c.sweeps[k];
    stats->device_ms = ms;
  }
  return status;
}

const void *persistent_kernel(int mode, bool halo) {
  if (halo) return mode == kMixed ? (const void *)ssa_persistent<kMixed, true> : (const void *)ssa_persistent<kFast64, true>;
  return mode == kMixed ? (const void *)ssa_persistent<kMixed, false>
         : mode == kFast64 ? (const void *)ssa_persistent<kFast64, false>
                           : (const void *)ssa_persistent<kExact64, false>;
}

}  // namespace
}  // namespace ufe

extern "C" int ufe_ssa_run(ufe_mesh_h h, const ufe_params *p, ufe_ssa_stats *stats) {
  if (!h || !p) { set_error("ufe_ssa_run: null argument"); return UFE_BAD_ARG; }
  SsaWork *w = h->ssa;
  if (!w || !w->uploaded) { set_error("ufe_ssa_run: no inputs uploaded"); return UFE_BAD_ARG; }
  int rc = check_params(p, "ufe_ssa_run");
  if (rc) return rc;
  cudaStream_t s = h->stream;
  std::memset(w->ctl_host, 0, sizeof(SsaCtl));
  rc = cuda_status(cudaEventRecord(w->ev0, s), "event");
  bool solve = false;
  SsaArgs a;
  if (!rc) rc = launch_prepare(h, p, s, &a, &solve);
  if (!rc && solve) {
    const int mode = sweep_mode(p);
    // Mirror each patch's own corrections in shared memory when the largest patch fits
    // (mixed sweeps: measured 34.3 against 35.2 us per sweep on the 200k-vertex dome; the
    // FP64 sweeps are bound by the FP64 pipe and gain nothing, so they keep plain loads).
    // UFE_SSA_LOCAL_ROWS=0 turns it off.
    const DevMesh &m = h->m;
    const size_t elem = mode == kMixed ? sizeof(float2) : sizeof(double2);
    // Halo sweeps when the mesh has the program and the largest working copy fits
    // (UFE_SSA_HALO=0 turns them off); else the phased sweeps with the optional mirror.
    const char *henv = std::getenv("UFE_SSA_HALO");
    // The parity (exact) mode keeps the phased sweeps: without fused multiply-adds it is bound
    // by the FP64 pipe, and the halo rows' extra updates measured slower there (133 against
    // 125 us per sweep on the 200k dome).
    const bool halo = m.has_halo && mode != kExact64 && (size_t)m.max_local * elem <= kLocalRowsMaxBytes &&
                      !(henv && henv[0] == '0');
    size_t bytes = halo ? (size_t)m.max_local * elem : (size_t)m.max_patch_slices * kSlice * elem;
    a.halo_index_off = (int)bytes;
    if (halo) bytes += (size_t)m.max_halo * sizeof(int);
    a.stage_off = (int)((bytes + 15) / 16 * 16);
    a.stage_bytes = 0;
    const char *env = std::getenv("UFE_SSA_LOCAL_ROWS");
    bool local = halo || (mode == kMixed && bytes <= kLocalRowsMaxBytes && !(env && env[0] == '0'));
    const void *fn = persistent_kernel(mode, halo);
    w->halo_used = halo;
    if (local) {
      // Ask for a shared-memory carveout that holds the mirror (the rest stays L1), and keep
      // the plain loads if one CTA per SM would then no longer fit.
      cudaFuncAttributes fa;
      int smem_sm = 0, per_sm = 0;
      rc = cuda_status(cudaFuncGetAttributes(&fa, fn), "function attributes");
      if (!rc) rc = cuda_status(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, h->device), "smem per SM");
      if (!rc && halo && mode == kMixed) {
        // the resident program slices take what one CTA per SM leaves of the shared memory
        int optin = 0;
        rc = cuda_status(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device), "smem opt-in");
        const long long room = (long long)optin - (long long)fa.sharedSizeBytes - (long long)a.stage_off - 1024;
        a.stage_bytes = room > 0 ? (int)(room / 16 * 16) : 0;
        bytes = (size_t)a.stage_off + (size_t)a.stage_bytes;
      }
      if (!rc) rc = cuda_status(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes), "smem attribute");
      const int pct = smem_sm > 0 ? (int)std::min<size_t>(100, (100 * (bytes + fa.sharedSizeBytes + 2048) + smem_sm - 1) / smem_sm) : 100;
      if (!rc) rc = cuda_status(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct), "carveout");
      if (!rc) rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, halo ? kHaloBlock : w->block, bytes), "occupancy");
      if (!rc && per_sm * h->num_sms < w->grid[mode]) {
        if (halo) { set_error("ufe_ssa_run: the halo sweeps' working copy leaves no room for one CTA per SM"); rc = UFE_CUDA_ERROR; }
        local = false;
      }
    }
    a.local_rows = local ? 1 : 0;
    const size_t smem = local ? bytes : 0;
    void *args[] = {(void *)&a};
    if (!rc)
      rc = cuda_status(cudaLaunchCooperativeKernel(fn, dim3(w->grid[mode]), dim3(halo ? kHaloBlock : w->block), args, smem, s),
                       "ssa_persistent");
  }
  if (!rc) rc = launch_finish(h, s);
  if (!rc) rc = cuda_status(cudaEventRecord(w->ev1, s), "event");
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "ssa solve");
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, w->ev0, w->ev1);
  return stats_of(*w->ctl_host, stats, ms);
}

extern "C" int ufe_ssa_download(ufe_mesh_h h, ufe_ssa_inout *io, ufe_ssa_out *out) {
  if (!h || !io) { set_error("ufe_ssa_download: null argument"); return UFE_BAD_ARG; }
  SsaWork *w = h->ssa;
  if (!w || !w->uploaded) { set_error("ufe_ssa_download: nothing solved"); return UFE_BAD_ARG; }
  const size_t nV = w->nV, nAc = w->nAc, nA = w->nA;
  cudaStream_t s = h->stream;
  const double *so = w->stage_out;
  int rc = d2h(io->U_SSA, so, nV, s);
  if (!rc) rc = d2h(io->V_SSA, so + nV, nV, s);
  if (!rc) rc = d2h(io->Ux_SSA_Ac, so + 2 * nV, nAc, s);
  if (!rc) rc = d2h(io->Uy_SSA_Ac, so + 2 * nV + nAc, nAc, s);
  const double *acb = so + 2 * nV + 2 * nAc;
  if (out) {
    if (!rc) rc = d2h(out->Up_SSA_Ac, acb, nAc, s);
    if (!rc) rc = d2h(out->Uo_SSA_Ac, acb + nAc, nAc, s);
  }
  const double *ab = acb + 2 * nAc;
  if (!rc && io->N_AaAc && !w->zero) rc = d2h(io->N_AaAc, ab, nA, s);
  if (out && !w->zero) {
    if (!rc) rc = d2h(out->eta_AaAc, ab + nA, nA, s);
    if (!rc) rc = d2h(out->S_AaAc, ab + 2 * nA, nA, s);
    if (!rc) rc = d2h(out->tau_c_AaAc, ab + 3 * nA, nA, s);
    if (!rc) rc = d2h(out->phi_fric_AaAc, ab + 4 * nA, nA, s);
  }
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "ssa download");
  return rc;
}

namespace ufe {
namespace {
// bottom_frictional_heating (thermodynamics_module.f90:281-311) on the Aa vertices, from the
// velocities and yield stress the last solve left in the staging buffer (caller order).
__global__ void k_frictional_heating(int nV, const int *mask_sheet, const double *tau, const double *U,
                                     const double *V, double *heating) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nV) return;
  double h = 0.0;
  if (mask_sheet[v] == 1) {
    const double delta_v = 1e-3, q_plastic = 0.30, u_threshold = 100.0;
    const double u = U[v], w = V[v];
    const double beta_base = (tau[v] * pow((delta_v * delta_v + u * u) + w * w, 0.5 * (q_plastic - 1.0))) /
                             pow(u_threshold, q_plastic);
    h = beta_base * (u * u + w * w);
  }
  heating[v] = h;
}
}  // namespace
}  // namespace ufe

extern "C" int ufe_ssa_frictional_heating(ufe_mesh_h h, const int32_t *mask_sheet, double *heating) {
  if (!h || !mask_sheet || !heating) { set_error("ufe_ssa_frictional_heating: null argument"); return UFE_BAD_ARG; }
  SsaWork *w = h->ssa;
  if (!w || !w->uploaded) { set_error("ufe_ssa_frictional_heating: no solve on this handle"); return UFE_BAD_ARG; }
  const size_t nV = w->nV, nAc = w->nAc, nA = w->nA;
  cudaStream_t s = h->stream;
  const double *so = w->stage_out;
  const double *tau = so + 2 * nV + 4 * nAc + 3 * nA;
  int rc = UFE_OK;
  if (!w->fh) rc = cuda_status(cudaMalloc(&w->fh, nV * (sizeof(double) + sizeof(int))), "frictional heating");
  if (rc) return rc;
  double *out = w->fh;
  int *mask = reinterpret_cast<int *>(w->fh + nV);
  rc = cuda_status(cudaMemcpyAsync(mask, mask_sheet, nV * sizeof(int), cudaMemcpyHostToDevice, s), "mask H2D");
  if (!rc) {
    k_frictional_heating<<<(unsigned)((nV + 255) / 256), 256, 0, s>>>((int)nV, mask, tau, so, so + nV, out);
    rc = cuda_status(cudaGetLastError(), "k_frictional_heating");
  }
  if (!rc) rc = d2h(heating, out, nV, s);
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "frictional heating");
  return rc;
}

extern "C" int ufe_ssa_solve(ufe_mesh_h h, const ufe_params *p, const ufe_ssa_in *in, ufe_ssa_inout *io,
                             ufe_ssa_out *out, ufe_ssa_stats *stats) {
  int rc = ufe_ssa_upload(h, p, in, io);
  if (rc < 0) return rc;
  const int status = ufe_ssa_run(h, p, stats);
  if (status < 0 && status != UFE_DIVERGED) return status;
  rc = ufe_ssa_download(h, io, out);
  if (rc < 0) return rc;
  return status;
}


// ---------------------------------------------------------------------------------------
// Batched ensemble: many independent solves in one persistent launch (no counterpart in
// the reference, whose model runs one solve_SSA per time step).
// ---------------------------------------------------------------------------------------
namespace ufe {
namespace {

constexpr int kMaxClasses = 16;
constexpr int kDefaultRowsPerCta = 8192;
// Largest rows per patch the planner allows: 3/4 of the per-CTA slice table (the rest is
// headroom for the padding of the six row groups to multiples of 32).
constexpr int kMaxRowsPerPatch = kMaxPatchSlices * kSlice * 3 / 4;

int pow2_ceil(int x) { int p = 1; while (p < x) p <<= 1; return p; }
int pow2_floor(int x) { int p = 1; while (2 * p <= x) p <<= 1; return p; }

// Estimated CTA-microseconds of a member solved by T CTAs of `block` threads: sqrt(rows)
// sweeps (the SOR count grows about like the mesh's linear resolution), each a latency
// floor plus a per-row cost that scales with the rows of a CTA.
double member_work(int rows, int T, int block) {
  const double sweeps = std::sqrt((double)rows);
  const double per_sweep_us = 20.0 + 0.0025 * (double)rows / T * (1024.0 / block);
  return (double)T * sweeps * per_sweep_us;
}

int plan_batch(const int32_t *rows, int n, const ufe_batch_config &cfg, int resident, int32_t *team_of_member,
               ufe_batch_plan_out *plan) {
  const int block = cfg.block ? cfg.block : 1024;
  if (resident < 1) { set_error("ufe_batch_plan: no co-resident CTAs"); return UFE_BAD_ARG; }
  for (int m = 0; m < n; ++m) {
    const int r = rows[m];
    if (r < 32) { set_error("ufe_batch_plan: member " + std::to_string(m) + " has fewer than 32 rows"); return UFE_BAD_ARG; }
    const int cap = std::min(resident, r / kSlice);           // patches of at least 32 rows
    const int need = (r + kMaxRowsPerPatch - 1) / kMaxRowsPerPatch;
    int T;
    if (cfg.team_ctas > 0) {
      T = cfg.team_ctas;
    } else {
      const int R = cfg.rows_per_cta > 0 ? cfg.rows_per_cta : kDefaultRowsPerCta;
      // Powers of two up to half the resident CTAs: one team of every class always fits
      // (1 + 2 + ... + 2^k = 2^(k+1) - 1).
      T = pow2_ceil(std::max(need, (r + R - 1) / R));
      T = std::min(T, pow2_floor(std::min(cap, (resident + 1) / 2)));
    }
    if (T > cap || T < need) {
      char buf[200];
      std::snprintf(buf, sizeof buf, "ufe_batch_plan: member %d (%d rows) cannot be cut into %d patches "
                                     "(between %d and %d fit)", m, r, T, need, cap);
      set_error(buf);
      return UFE_BAD_ARG;
    }
    team_of_member[m] = T;
  }
  // Classes: distinct team sizes, largest first.
  std::vector<int> sizes(team_of_member, team_of_member + n);
  std::sort(sizes.begin(), sizes.end(), std::greater<int>());
  sizes.erase(std::unique(sizes.begin(), sizes.end()), sizes.end());
  if ((int)sizes.size() > kMaxClasses) { set_error("ufe_batch_plan: too many team sizes"); return UFE_BAD_ARG; }
  const int nc = (int)sizes.size();
  std::vector<double> W(nc, 0.0);
  std::vector<int> members(nc, 0), teams(nc, 0);
  double Wt = 0.0;
  for (int m = 0; m < n; ++m) {
    const int c = (int)(std::find(sizes.begin(), sizes.end(), team_of_member[m]) - sizes.begin());
    const double w = member_work(rows[m], team_of_member[m], block);
    W[c] += w;
    Wt += w;
    members[c] += 1;
  }
  // CTAs to each class in proportion to its work, at least one team per class.
  int used = 0;
  for (int c = 0; c < nc; ++c) {
    teams[c] = std::max(1, std::min(members[c], (int)std::floor(resident * W[c] / Wt / sizes[c])));
    used += teams[c] * sizes[c];
  }
  while (used > resident) {   // over-subscribed: take a team from the most generously served class
    int best = -1;
    double r = -1.0;
    for (int c = 0; c < nc; ++c)
      if (teams[c] > 1 && teams[c] * sizes[c] / W[c] > r) { r = teams[c] * sizes[c] / W[c]; best = c; }
    if (best < 0) { set_error("ufe_batch_plan: the team sizes need more CTAs than the device holds"); return UFE_BAD_ARG; }
    teams[best] -= 1;
    used -= sizes[best];
  }
  for (;;) {                  // spare CTAs: give a team to the least served class that can use it
    int best = -1;
    double r = 1e300;
    for (int c = 0; c < nc; ++c)
      if (teams[c] < members[c] && used + sizes[c] <= resident && teams[c] * sizes[c] / W[c] < r) {
        r = teams[c] * sizes[c] / W[c];
        best = c;
      }
    if (best < 0) break;
    teams[best] += 1;
    used += sizes[best];
  }
  std::memset(plan, 0, sizeof(*plan));
  plan->n_classes = nc;
  for (int c = 0; c < nc; ++c) { plan->class_team_ctas[c] = sizes[c]; plan->class_teams[c] = teams[c]; }
  plan->grid_ctas = used;
  return UFE_OK;
}

}  // namespace
}  // namespace ufe

struct ufe_batch_s {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int n = 0;                          // members
  int block = 0;                      // threads per CTA of the batched kernel
  bool use_graph = true;
  // mixed members on the halo sweeps: every member has the program and the largest working copy
  // (plus halo indices) fits the CTAs the plan keeps resident
  bool halo_ok = false;
  int halo_index_off = 0, halo_stage_off = 0;
  size_t halo_smem = 0;
  ufe_batch_plan_out plan{};
  int n_teams = 0;
  std::vector<int32_t> team_of_member;
  std::vector<ufe_mesh_h> members;    // owned
  std::vector<double> cost;           // expected relative cost of each member
  std::vector<int> order;             // queue position -> member (active members only)
  SsaArgs *args_host = nullptr;       // pinned, [n] by queue position
  SsaArgs *args_dev = nullptr;
  int *layout_host = nullptr;         // pinned: team_of_cta, team_info (int4), class_range (int2)
  int *layout_dev = nullptr;
  size_t layout_words = 0;
  unsigned int *sched = nullptr;      // queues (32 words per class), team_bar, team_member
  size_t sched_words = 0;
  unsigned long long *times_dev = nullptr, *times_host = nullptr;   // [2n]
  int *err_dev = nullptr, *err_host = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ufe_params graph_params{};          // what the graph was captured for
  std::vector<uint8_t> graph_flags;   // per member: uploaded state the graph depends on
};

namespace ufe {
namespace {

void batch_free(ufe_batch_s *b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (ufe_mesh_h h : b->members)
    if (h) ufe_mesh_destroy(h);
  void *host[] = {b->args_host, b->times_host, b->err_host, b->layout_host};
  for (void *p : host)
    if (p) cudaFreeHost(p);
  void *dev[] = {b->args_dev, b->sched, b->times_dev, b->err_dev, b->layout_dev};
  for (void *p : dev)
    if (p) cudaFree(p);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// The batched kernel for a sweep mode and CTA shape (nullptr: not built); halo: the mixed
// members' halo sweeps.
const void *batched_kernel(int mode, int block, bool halo = false) {
  if (halo) {
    switch (mode * 10000 + block) {
      case kMixed * 10000 + 1024: return (const void *)ssa_batched<kMixed, 1024, 1, true>;
      case kMixed * 10000 + 512: return (const void *)ssa_batched<kMixed, 512, 2, true>;
      case kMixed * 10000 + 256: return (const void *)ssa_batched<kMixed, 256, 4, true>;
      default: return nullptr;
    }
  }
  switch (mode * 10000 + block) {
    case kExact64 * 10000 + 1024: return (const void *)ssa_batched<kExact64, 1024, 1>;
    case kFast64 * 10000 + 1024: return (const void *)ssa_batched<kFast64, 1024, 1>;
    case kFast64 * 10000 + 512: return (const void *)ssa_batched<kFast64, 512, 2>;
    case kFast64 * 10000 + 256: return (const void *)ssa_batched<kFast64, 256, 4>;
    case kMixed * 10000 + 1024: return (const void *)ssa_batched<kMixed, 1024, 1>;
    case kMixed * 10000 + 512: return (const void *)ssa_batched<kMixed, 512, 2>;
    case kMixed * 10000 + 256: return (const void *)ssa_batched<kMixed, 256, 4>;
    default: return nullptr;
  }
}

// Raises a batched kernel's dynamic shared-memory limit on a device to at least `bytes`, never
// lowering it (batches alive at the same time share the kernel, and a captured batch replays with
// the size it was captured with); false when the device cannot give that much.
bool raise_dynamic_smem(const void *fn, int device, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> limit;
  std::lock_guard<std::mutex> lock(mu);
  size_t &cur = limit[std::make_pair(device, fn)];
  if (bytes <= cur) return true;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cur = bytes;
  return true;
}

// Co-resident CTAs of the batched kernels of one CTA size (the smallest over the modes).
int resident_ctas(int block, int num_sms, int *out) {
  int per_sm = 1 << 30;
  for (int mode = 0; mode < 3; ++mode) {
    const void *fn = batched_kernel(mode, block);
    if (!fn) continue;
    int q = 0;
    const int rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, fn, block, 0), "occupancy");
    if (rc) return rc;
    per_sm = std::min(per_sm, q);
  }
  *out = per_sm * num_sms;
  return UFE_OK;
}

uint8_t member_flags(ufe_mesh_h h) {
  const SsaWork *w = h->ssa;
  if (!w) return 0;
  return (uint8_t)(1 | (w->has_beta << 1) | (w->has_N << 2) | (w->gl << 3) | (w->zero << 4) | (w->uploaded << 5));
}

bool same_params(const ufe_params &a, const ufe_params &b) {
  return a.SSA_RN_tol == b.SSA_RN_tol && a.SSA_max_outer_loops == b.SSA_max_outer_loops &&
         a.SSA_max_residual_UV == b.SSA_max_residual_UV && a.SSA_SOR_omega == b.SSA_SOR_omega &&
         a.SSA_max_inner_loops == b.SSA_max_inner_loops && a.m_enh_ssa == b.m_enh_ssa &&
         a.sliding_law == b.sliding_law && a.beta_sq == b.beta_sq &&
         a.use_analytical_GL_flux == b.use_analytical_GL_flux && a.zero_velocities == b.zero_velocities &&
         a.precision == b.precision && a.mixed_refold_sweeps == b.mixed_refold_sweeps &&
         a.fp64_exact == b.fp64_exact && a.mixed_fp32_viscosity == b.mixed_fp32_viscosity;
}

// Enqueue one whole batch on b->stream: per member gather (and GL flux), the persistent
// batched solve over the active members, per member scatter and control-block read-back.
int batch_enqueue(ufe_batch_s *b, const ufe_params *p, int mode) {
  cudaStream_t s = b->stream;
  const ufe_batch_plan_out &pl = b->plan;
  const int nc = pl.n_classes;
  b->order.clear();
  int rc = UFE_OK;
  // Queue order: by class (largest teams first), then by expected cost.
  std::vector<int> by(b->n);
  std::iota(by.begin(), by.end(), 0);
  std::stable_sort(by.begin(), by.end(), [&](int x, int y) {
    if (b->team_of_member[x] != b->team_of_member[y]) return b->team_of_member[x] > b->team_of_member[y];
    return b->cost[x] > b->cost[y];
  });
  int *tc = b->layout_host;                                     // team_of_cta [grid]
  int4 *ti = reinterpret_cast<int4 *>(tc + ((pl.grid_ctas + 3) & ~3));   // [n_teams]
  int2 *cr = reinterpret_cast<int2 *>(ti + b->n_teams);         // [n_classes]
  for (int c = 0; c < nc; ++c) cr[c] = make_int2(0, 0);
  for (int k = 0; k < b->n && !rc; ++k) {
    const int m = by[k];
    bool solve = false;
    SsaArgs a;
    rc = launch_prepare(b->members[m], p, s, &a, &solve);
    if (!rc && solve && mode == kMixed && b->halo_ok) {
      a.halo_index_off = b->halo_index_off;
      a.stage_off = b->halo_stage_off;
      a.stage_bytes = 0;
    }
    if (!rc && solve) {
      const int c = (int)(std::find(pl.class_team_ctas, pl.class_team_ctas + nc, b->team_of_member[m]) -
                          pl.class_team_ctas);
      const int q = (int)b->order.size();
      if (cr[c].y == cr[c].x) cr[c] = make_int2(q, q);
      cr[c].y = q + 1;
      b->args_host[q] = a;
      b->order.push_back(m);
    }
  }
  const int n_active = (int)b->order.size();
  // Team layout: teams of class 0 first, CTAs of a team contiguous.
  int team = 0, cta = 0;
  for (int c = 0; c < nc; ++c)
    for (int k = 0; k < pl.class_teams[c]; ++k, ++team) {
      ti[team] = make_int4(cta, pl.class_team_ctas[c], c, 0);
      for (int r = 0; r < pl.class_team_ctas[c]; ++r) tc[cta++] = team;
    }
  const void *fn = batched_kernel(mode, b->block);   // (the halo variant below when it applies)
  if (!rc && n_active > 0) {
    unsigned int *queue = b->sched, *team_bar = queue + 32 * (size_t)kMaxClasses;
    unsigned int *team_member = team_bar + 32 * (size_t)b->n_teams;
    rc = cuda_status(cudaMemsetAsync(b->sched, 0, b->sched_words * sizeof(unsigned int), s), "memset sched");
    if (!rc) rc = cuda_status(cudaMemsetAsync(b->err_dev, 0, sizeof(int), s), "memset err");
    if (!rc) rc = cuda_status(cudaMemsetAsync(b->times_dev, 0, 2 * (size_t)b->n * sizeof(unsigned long long), s), "memset times");
    if (!rc)
      rc = cuda_status(cudaMemcpyAsync(b->args_dev, b->args_host, (size_t)n_active * sizeof(SsaArgs),
                                       cudaMemcpyHostToDevice, s), "args H2D");
    if (!rc)
      rc = cuda_status(cudaMemcpyAsync(b->layout_dev, b->layout_host, b->layout_words * sizeof(int),
                                       cudaMemcpyHostToDevice, s), "layout H2D");
    const int *tcd = b->layout_dev;
    const int4 *tid = reinterpret_cast<const int4 *>(tcd + ((pl.grid_ctas + 3) & ~3));
    BatchArgs ba;
    ba.members = b->args_dev; ba.n_members = n_active;
    ba.team_of_cta = tcd; ba.team_info = tid; ba.class_range = reinterpret_cast<const int2 *>(tid + b->n_teams);
    ba.queue = queue; ba.team_bar = team_bar; ba.team_member = team_member;
    ba.times = b->times_dev; ba.err = b->err_dev; ba.timeout_ns = wait_timeout_ns();
    const bool halo = mode == kMixed && b->halo_ok;
    if (halo) fn = batched_kernel(mode, b->block, true);
    if (!rc) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)pl.grid_ctas);
      cfg.blockDim = dim3((unsigned)b->block);
      cfg.dynamicSmemBytes = halo ? b->halo_smem : 0;
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      void *kargs[] = {(void *)&ba};
      rc = cuda_status(cudaLaunchKernelExC(&cfg, fn, kargs), "ssa_batched");
    }
  }
  for (int m = 0; m < b->n && !rc; ++m) rc = launch_finish(b->members[m], s);
  if (!rc)
    rc = cuda_status(cudaMemcpyAsync(b->times_host, b->times_dev, 2 * (size_t)b->n * sizeof(unsigned long long),
                                     cudaMemcpyDeviceToHost, s), "times D2H");
  if (!rc) rc = cuda_status(cudaMemcpyAsync(b->err_host, b->err_dev, sizeof(int), cudaMemcpyDeviceToHost, s), "err D2H");
  return rc;
}

int check_block(const ufe_batch_config *cfg, int *block, const char *who) {
  *block = cfg && cfg->block ? cfg->block : 1024;
  if (*block != 1024 && *block != 512 && *block != 256) {
    set_error(std::string(who) + ": block must be 1024, 512 or 256 threads");
    return UFE_BAD_ARG;
  }
  if (cfg && (cfg->team_ctas < 0 || cfg->rows_per_cta < 0)) {
    set_error(std::string(who) + ": team_ctas and rows_per_cta must be >= 0");
    return UFE_BAD_ARG;
  }
  return UFE_OK;
}

}  // namespace
}  // namespace ufe

extern "C" int ufe_batch_plan(const int32_t *rows, int32_t n, const ufe_batch_config *cfg, int32_t resident,
                              int32_t *team_ctas_of_member, ufe_batch_plan_out *plan) {
  if (!rows || n < 1 || !team_ctas_of_member || !plan) { set_error("ufe_batch_plan: null argument"); return UFE_BAD_ARG; }
  int block = 0;
  int rc = check_block(cfg, &block, "ufe_batch_plan");
  if (rc) return rc;
  ufe_batch_config c = cfg ? *cfg : ufe_batch_config{};
  c.block = block;
  return plan_batch(rows, n, c, resident, team_ctas_of_member, plan);
}

extern "C" int ufe_batch_create(const ufe_mesh_desc *descs, int32_t n, const ufe_batch_config *cfg,
                                ufe_batch_h *out) {
  if (!descs || !out || n < 1) { set_error("ufe_batch_create: null argument or no members"); return UFE_BAD_ARG; }
  *out = nullptr;
  int block = 0;
  int rc = check_block(cfg, &block, "ufe_batch_create");
  if (rc) return rc;
  ufe_batch_s *b = new ufe_batch_s();
  b->n = n; b->block = block; b->use_graph = !cfg || cfg->use_graph != 0;
  rc = cuda_status(cudaGetDevice(&b->device), "cudaGetDevice");
  if (!rc) rc = cuda_status(cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device), "SM count");
  int resident = 0;
  if (!rc) rc = resident_ctas(block, b->num_sms, &resident);
  std::vector<int32_t> rows(n);
  for (int k = 0; k < n; ++k) rows[k] = descs[k].nVAaAc;
  b->team_of_member.assign(n, 0);
  if (!rc) {
    ufe_batch_config c = cfg ? *cfg : ufe_batch_config{};
    c.block = block;
    rc = plan_batch(rows.data(), n, c, resident, b->team_of_member.data(), &b->plan);
  }
  if (!rc) rc = cuda_status(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  b->members.assign(n, nullptr);
  b->cost.assign(n, 0.0);
  for (int k = 0; k < n && !rc; ++k) {
    rc = mesh_create(descs + k, b->team_of_member[k], &b->members[k]);
    if (!rc && b->members[k]->m.n_patch != b->team_of_member[k]) {
      set_error("ufe_batch_create: member " + std::to_string(k) + " has too few rows for its team");
      rc = UFE_BAD_ARG;
    } else if (rc) {
      const std::string e = ufe_last_error_string();
      set_error("ufe_batch_create: member " + std::to_string(k) + ": " + e);
    }
    if (!rc) b->cost[k] = member_work(rows[k], 1, 1024);
  }
  if (!rc) {
    // Mixed members run the halo sweeps when every member has the program and the largest working
    // copy with its halo indices leaves the plan's CTAs co-resident (else the phased sweeps).
    int max_local = 0, max_halo = 0;
    bool all = true;
    for (ufe_mesh_h h : b->members) {
      all = all && h->m.has_halo;
      max_local = std::max(max_local, h->m.max_local);
      max_halo = std::max(max_halo, h->m.max_halo);
    }
    const void *fn = batched_kernel(kMixed, block, true);
    if (all && fn) {
      const size_t idx_off = (size_t)max_local * sizeof(float2);
      const size_t stage_off = (idx_off + (size_t)max_halo * sizeof(int) + 15) / 16 * 16;
      int per_sm = 0;
      if (raise_dynamic_smem(fn, b->device, stage_off) &&
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, stage_off) == cudaSuccess &&
          per_sm * b->num_sms >= b->plan.grid_ctas) {
        b->halo_ok = true;
        b->halo_index_off = (int)idx_off;
        b->halo_stage_off = (int)stage_off;
        b->halo_smem = stage_off;
      } else {
        cudaGetLastError();   // a working copy too large for the device: the phased sweeps
      }
    }
  }
  if (!rc) {
    b->n_teams = 0;
    for (int c = 0; c < b->plan.n_classes; ++c) b->n_teams += b->plan.class_teams[c];
    b->layout_words = (size_t)((b->plan.grid_ctas + 3) & ~3) + 4 * (size_t)b->n_teams + 2 * (size_t)kMaxClasses;
    b->sched_words = 32 * (size_t)kMaxClasses + 64 * (size_t)b->n_teams;
  }
  if (!rc) rc = cuda_status(cudaMallocHost(&b->args_host, (size_t)n * sizeof(SsaArgs)), "batch args host");
  if (!rc) rc = cuda_status(cudaMalloc(&b->args_dev, (size_t)n * sizeof(SsaArgs)), "batch args");
  if (!rc) rc = cuda_status(cudaMallocHost(&b->layout_host, b->layout_words * sizeof(int)), "batch layout host");
  if (!rc) rc = cuda_status(cudaMalloc(&b->layout_dev, b->layout_words * sizeof(int)), "batch layout");
  if (!rc) rc = cuda_status(cudaMalloc(&b->sched, b->sched_words * sizeof(unsigned int)), "batch sched");
  if (!rc) rc = cuda_status(cudaMalloc(&b->times_dev, 2 * (size_t)n * sizeof(unsigned long long)), "batch times");
  if (!rc) rc = cuda_status(cudaMallocHost(&b->times_host, 2 * (size_t)n * sizeof(unsigned long long)), "batch times host");
  if (!rc) rc = cuda_status(cudaMalloc(&b->err_dev, sizeof(int)), "batch err");
  if (!rc) rc = cuda_status(cudaMallocHost(&b->err_host, sizeof(int)), "batch err host");
  if (!rc) rc = cuda_status(cudaEventCreate(&b->ev0), "event");
  if (!rc) rc = cuda_status(cudaEventCreate(&b->ev1), "event");
  if (rc) { batch_free(b); return rc; }
  *out = b;
  return UFE_OK;
}

extern "C" int ufe_batch_destroy(ufe_batch_h b) {
  if (!b) return UFE_BAD_ARG;
  cudaStreamSynchronize(b->stream);
  batch_free(b);
  return UFE_OK;
}

extern "C" int ufe_batch_upload(ufe_batch_h b, int32_t member, const ufe_params *p, const ufe_ssa_in *in,
                                const ufe_ssa_inout *io) {
  if (!b || member < 0 || member >= b->n) { set_error("ufe_batch_upload: bad batch or member index"); return UFE_BAD_ARG; }
  ufe_mesh_h h = b->members[member];
  int rc = ufe_ssa_upload(h, p, in, io);
  if (!rc) rc = cuda_status(cudaStreamSynchronize(h->stream), "batch upload");
  return rc;
}

extern "C" int ufe_batch_download(ufe_batch_h b, int32_t member, ufe_ssa_inout *io, ufe_ssa_out *out) {
  if (!b || member < 0 || member >= b->n) { set_error("ufe_batch_download: bad batch or member index"); return UFE_BAD_ARG; }
  return ufe_ssa_download(b->members[member], io, out);
}

extern "C" int ufe_batch_run(ufe_batch_h b, const ufe_params *p, ufe_ssa_stats *stats, ufe_batch_timing *timing) {
  if (!b || !p) { set_error("ufe_batch_run: null argument"); return UFE_BAD_ARG; }
  int rc = check_params(p, "ufe_batch_run");
  if (rc) return rc;
  for (int m = 0; m < b->n; ++m)
    if (!b->members[m]->ssa || !b->members[m]->ssa->uploaded) {
      set_error("ufe_batch_run: member " + std::to_string(m) + " has no uploaded inputs");
      return UFE_BAD_ARG;
    }
  const int mode = sweep_mode(p);
  if (!batched_kernel(mode, b->block)) {
    set_error("ufe_batch_run: the exact FP64 mode is built for 1024-thread CTAs only");
    return UFE_BAD_ARG;
  }
  cudaStream_t s = b->stream;
  for (int m = 0; m < b->n; ++m) std::memset(b->members[m]->ssa->ctl_host, 0, sizeof(SsaCtl));
  *b->err_host = 0;
  if (b->use_graph) {
    // Captured once per parameter set and upload state; a replay re-runs every step,
    // including the gathers of the currently uploaded inputs.
    std::vector<uint8_t> flags(b->n);
    for (int m = 0; m < b->n; ++m) flags[m] = member_flags(b->members[m]);
    if (!b->exec || !same_params(b->graph_params, *p) || flags != b->graph_flags) {
      if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
      if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
      rc = cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
      if (!rc) {
        const int rc_enq = batch_enqueue(b, p, mode);
        const int rc_end = cuda_status(cudaStreamEndCapture(s, &b->graph), "end capture");
        rc = rc_enq ? rc_enq : rc_end;
      }
      if (!rc) rc = cuda_status(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
      if (rc) return rc;
      b->graph_params = *p;
      b->graph_flags = flags;
    }
    rc = cuda_status(cudaEventRecord(b->ev0, s), "event");
    if (!rc) rc = cuda_status(cudaGraphLaunch(b->exec, s), "graph launch");
  } else {
    rc = cuda_status(cudaEventRecord(b->ev0, s), "event");
    if (!rc) rc = batch_enqueue(b, p, mode);
  }
  if (!rc) rc = cuda_status(cudaEventRecord(b->ev1, s), "event");
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "batch solve");
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  int worst = UFE_OK;
  for (int m = 0; m < b->n; ++m) {
    const int st = stats_of(*b->members[m]->ssa->ctl_host, stats ? stats + m : nullptr, ms);
    if (st < 0 && (worst >= 0 || st < worst)) worst = st;
    else if (worst >= 0 && st > worst) worst = st;
  }
  if (*b->err_host && worst >= 0) {
    worst = *b->err_host;
    set_error("ufe_batch_run: a device-side bounded wait timed out");
  }
  if (timing) {
    const int n_active = (int)b->order.size();
    std::vector<double> dur;
    unsigned long long t0 = ~0ull, t1 = 0ull;
    for (int q = 0; q < n_active; ++q) {
      const unsigned long long a = b->times_host[2 * q], e = b->times_host[2 * q + 1];
      if (e > a) {
        dur.push_back(1e-6 * (double)(e - a));
        t0 = std::min(t0, a);
        t1 = std::max(t1, e);
        if (timing->member_ms) timing->member_ms[b->order[q]] = 1e-6 * (double)(e - a);
      }
    }
    std::sort(dur.begin(), dur.end());
    auto pct = [&](double f) {   // nearest-rank percentile
      if (dur.empty()) return 0.0;
      const long r = (long)std::ceil(f * (double)dur.size()) - 1;
      return dur[(size_t)std::min<long>((long)dur.size() - 1, std::max<long>(0, r))];
    };
    timing->device_ms = ms;
    timing->solve_ms = t1 > t0 ? 1e-6 * (double)(t1 - t0) : 0.0;
    timing->member_p50_ms = pct(0.5);
    timing->member_p99_ms = pct(0.99);
    timing->member_max_ms = dur.empty() ? 0.0 : dur.back();
    timing->n_active = n_active;
    timing->n_teams = b->n_teams;
    timing->n_classes = b->plan.n_classes;
    timing->grid_ctas = b->plan.grid_ctas;
    timing->max_team_ctas = b->plan.class_team_ctas[0];
    timing->block = b->block;
  }
  return worst;
}

extern "C" int ufe_ssa_solve_batched(int32_t n, const ufe_mesh_desc *descs, const ufe_batch_config *cfg,
                                     const ufe_params *p, const ufe_ssa_in *in, ufe_ssa_inout *io, ufe_ssa_out *out,
                                     ufe_ssa_stats *stats) {
  if (!descs || !p || !in || !io || n < 1) { set_error("ufe_ssa_solve_batched: null argument"); return UFE_BAD_ARG; }
  ufe_batch_h b = nullptr;
  int rc = ufe_batch_create(descs, n, cfg, &b);
  for (int m = 0; m < n && !rc; ++m) rc = ufe_batch_upload(b, m, p, in + m, io + m);
  int status = UFE_OK;
  if (!rc) {
    status = ufe_batch_run(b, p, stats, nullptr);
    if (status < 0 && status != UFE_DIVERGED) rc = status;
  }
  for (int m = 0; m < n && !rc; ++m) rc = ufe_batch_download(b, m, io + m, out ? out + m : nullptr);
  if (b) ufe_batch_destroy(b);
  return rc ? rc : status;
}

// Autotuner of the batched solve: the per-CTA packing (rows_per_cta, hence the team size of
// every member) first at 1024-thread CTAs, then the CTA size at the best packing, then the
// neighbouring packings at the best CTA size. Each
// candidate is a real batch of the caller's members, solved twice (the first run captures
// the graph); the second run's device time decides.
extern "C" int ufe_batch_autotune(int32_t n, const ufe_mesh_desc *descs, const ufe_params *p, const ufe_ssa_in *in,
                                  const ufe_ssa_inout *io, ufe_batch_config *best, ufe_batch_tune_entry *log,
                                  int32_t log_capacity, int32_t *log_count) {
  if (!descs || !p || !in || !io || !best || n < 1) { set_error("ufe_batch_autotune: null argument"); return UFE_BAD_ARG; }
  int n_log = 0;
  double best_ms = 1e300;
  ufe_batch_config best_cfg{0, kDefaultRowsPerCta, 1024, 1};
  auto trial = [&](const ufe_batch_config &c) -> int {
    ufe_batch_h b = nullptr;
    int rc = ufe_batch_create(descs, n, &c, &b);
    if (rc == UFE_BAD_ARG) return UFE_OK;   // this packing does not fit these members: skip it
    for (int m = 0; m < n && !rc; ++m) rc = ufe_batch_upload(b, m, p, in + m, io + m);
    ufe_batch_timing t{};
    for (int k = 0; k < 2 && !rc; ++k) {
      const int st = ufe_batch_run(b, p, nullptr, &t);
      if (st < 0 && st != UFE_DIVERGED) rc = st;
    }
    if (b) ufe_batch_destroy(b);
    if (rc) return rc;
    if (log && n_log < log_capacity) {
      log[n_log].rows_per_cta = c.rows_per_cta;
      log[n_log].block = c.block;
      log[n_log].grid_ctas = t.grid_ctas;
      log[n_log].n_classes = t.n_classes;
      log[n_log].device_ms = t.device_ms;
      log[n_log].member_p99_ms = t.member_p99_ms;
    }
    ++n_log;
    if (t.device_ms < best_ms) { best_ms = t.device_ms; best_cfg = c; }
    return UFE_OK;
  };
  int rc = UFE_OK;
  const int packings[] = {4096, 8192, 16384, kMaxRowsPerPatch};
  const int n_pack = 4;
  for (int R : packings)
    if (!rc) rc = trial(ufe_batch_config{0, R, 1024, 1});
  const int R = best_cfg.rows_per_cta;
  for (int blk : {512, 256})
    if (!rc) rc = trial(ufe_batch_config{0, R, blk, 1});
  // The packings next to the best one at the best CTA size.
  const int blk = best_cfg.block;
  if (blk != 1024) {
    const int i = (int)(std::find(packings, packings + n_pack, R) - packings);
    for (int j : {i - 1, i + 1})
      if (!rc && j >= 0 && j < n_pack) rc = trial(ufe_batch_config{0, packings[j], blk, 1});
  }
  if (log_count) *log_count = n_log;
  if (rc) return rc;
  if (best_ms == 1e300) { set_error("ufe_batch_autotune: no candidate fits these members"); return UFE_BAD_ARG; }
  *best = best_cfg;
  return UFE_OK;
}

// ---------------------------------------------------------------------------------------
// VJP of the converged solve (no counterpart in the reference)
// ---------------------------------------------------------------------------------------
namespace ufe {

struct AdjWork {
  int nP = 0, nV = 0, nAc = 0, nA = 0;
  int64_t nE = 0;
  double2 *cT = nullptr, *kT = nullptr;
  double2 *ee = nullptr, *kh = nullptr, *alpha = nullptr, *dinv = nullptr, *g = nullptr, *mu = nullptr;
  double *c3 = nullptr, *s = nullptr, *eta = nullptr, *fr = nullptr, *inv_nb = nullptr, *K = nullptr;
  double *stage = nullptr;        // dJ/du in (4 blocks), sensitivities out (6 nA), dHi (nV), dJ/dphi (nA)
  int *geom_int = nullptr;        // nC, C, Aci
  double *geom_dbl = nullptr;     // Nx, Ny, Nx_Ac, Ny_Ac
  unsigned int *prog = nullptr;
  AdjCtl *ctl = nullptr;
  AdjCtl *ctl_host = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // Krylov work (allocated on first use): basis (restart + 1 vectors), w, x, c, zero rows,
  // dot partials (device and pinned host), Givens coefficients on the device
  double *kry = nullptr;
  size_t kry_vectors = 0;
  double *part = nullptr, *part_host = nullptr, *hdev = nullptr;
};

void adj_free(AdjWork *w) {
  if (!w) return;
  void *ptrs[] = {w->cT, w->kT, w->ee, w->kh, w->alpha, w->dinv, w->g, w->mu, w->c3, w->s, w->eta, w->fr,
                  w->inv_nb, w->K, w->stage, w->geom_int, w->geom_dbl, w->prog, w->ctl, w->kry, w->part, w->hdev};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (w->ctl_host) cudaFreeHost(w->ctl_host);
  if (w->part_host) cudaFreeHost(w->part_host);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  delete w;
}

namespace {

int ensure_adj(ufe_mesh_h h) {
  if (h->adj) return UFE_OK;
  const DevMesh &m = h->m;
  AdjWork *w = new AdjWork();
  w->nP = m.nP; w->nV = m.nV; w->nAc = m.nAc; w->nA = m.nA; w->nE = m.nE;
  const size_t nP = m.nP, nE = (size_t)m.nE, nA = m.nA, nV = m.nV, nAc = m.nAc, ncm = m.ncm;
  int rc = cuda_status(cudaMalloc(&w->cT, nE * sizeof(double2)), "adj cT");
  if (!rc) rc = cuda_status(cudaMalloc(&w->kT, nE * sizeof(double2)), "adj kT");
  double2 **d2[] = {&w->ee, &w->kh, &w->alpha, &w->dinv, &w->g, &w->mu};
  for (double2 **q : d2)
    if (!rc) rc = cuda_status(cudaMalloc(q, nP * sizeof(double2)), "adj rows");
  double **d1[] = {&w->c3, &w->s, &w->eta, &w->fr, &w->inv_nb};
  for (double **q : d1)
    if (!rc) rc = cuda_status(cudaMalloc(q, nP * sizeof(double)), "adj rows");
  if (!rc) rc = cuda_status(cudaMalloc(&w->K, 3 * nP * sizeof(double)), "adj strain");
  if (!rc) rc = cuda_status(cudaMalloc(&w->stage, (2 * nV + 2 * nAc + 7 * nA + nV) * sizeof(double)), "adj stage");
  if (!rc) rc = cuda_status(cudaMalloc(&w->geom_int, (nV + nV * ncm + 4 * nAc) * sizeof(int)), "adj geom");
  if (!rc) rc = cuda_status(cudaMalloc(&w->geom_dbl, (2 * nV * (ncm + 1) + 8 * nAc) * sizeof(double)), "adj geom");
  if (!rc) rc = cuda_status(cudaMalloc(&w->prog, 32 * (size_t)m.n_patch * sizeof(unsigned int)), "adj progress");
  if (!rc) rc = cuda_status(cudaMalloc(&w->ctl, sizeof(AdjCtl)), "adj ctl");
  if (!rc) rc = cuda_status(cudaMallocHost(&w->ctl_host, sizeof(AdjCtl)), "adj ctl host");
  if (!rc) rc = cuda_status(cudaEventCreate(&w->ev0), "event");
  if (!rc) rc = cuda_status(cudaEventCreate(&w->ev1), "event");
  if (!rc) {
    int per_sm = 0;
    rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)ssa_adjoint_sor, kSsaBlock, 0),
                     "occupancy");
    if (!rc && per_sm * h->num_sms < m.n_patch) {
      set_error("ssa adjoint: not enough co-resident CTAs for one per patch");
      rc = UFE_CUDA_ERROR;
    }
  }
  if (rc) { adj_free(w); return rc; }
  h->adj = w;
  return UFE_OK;
}

}  // namespace
}  // namespace ufe

namespace ufe {
namespace {

constexpr int kKrylovBlocks = 304;

struct Krylov {
  int sweeps_per_apply = 1;
  ufe_mesh_h h;
  AdjWork *a;
  AdjArgs aa;
  cudaStream_t s;
  int nP, n;          // rows, vector length (2 nP)
  size_t ld;          // vector stride
  double *V, *w, *x, *c;
  double2 *zero;
  int sweeps = 0;
  int err = 0;
};

// One transposed sweep of mu (in place) with right-hand side g.
int kry_sweep(Krylov &k, const double2 *g) {
  int rc = cuda_status(cudaMemsetAsync(k.a->prog, 0, 32 * (size_t)k.h->m.n_patch * sizeof(unsigned int), k.s), "memset prog");
  if (!rc) rc = cuda_status(cudaMemsetAsync(k.a->ctl, 0, sizeof(AdjCtl), k.s), "memset adj ctl");
  AdjArgs aa = k.aa;
  aa.g = g;
  aa.max_sweeps = k.sweeps_per_apply;
  aa.tol = 0.0;
  void *args[] = {(void *)&aa};
  if (!rc)
    rc = cuda_status(cudaLaunchCooperativeKernel((const void *)ssa_adjoint_sor, dim3(k.h->m.n_patch), dim3(kSsaBlock), args, 0, k.s),
                     "ssa_adjoint_sor");
  k.sweeps += k.sweeps_per_apply;
  return rc;
}

// y = x - S(x; 0)
int kry_apply(Krylov &k, const double *xin, double *y) {
  const unsigned gp = (unsigned)((k.nP + 255) / 256), gn = (unsigned)((k.n + 255) / 256);
  k_krylov_load<<<gp, 256, 0, k.s>>>(k.nP, reinterpret_cast<const double2 *>(xin), k.a->alpha, k.a->mu, k.a->s);
  int rc = cuda_status(cudaGetLastError(), "k_krylov_load");
  if (!rc) rc = kry_sweep(k, k.zero);
  if (!rc) {
    k_krylov_sub<<<gn, 256, 0, k.s>>>(k.n, xin, reinterpret_cast<const double *>(k.a->mu), y);
    rc = cuda_status(cudaGetLastError(), "k_krylov_sub");
  }
  return rc;
}

// h[i] = V_i . wv for i < nvec (fixed-order sums: deterministic); also reads back the
// sweep control block so that a failed wait is noticed.
int kry_dots(Krylov &k, int nvec, const double *Vb, const double *wv, double *hout) {
  k_krylov_dots<<<dim3(kKrylovBlocks, nvec), 256, 0, k.s>>>(k.n, Vb, k.ld, wv, k.a->part);
  int rc = cuda_status(cudaGetLastError(), "k_krylov_dots");
  if (!rc)
    rc = cuda_status(cudaMemcpyAsync(k.a->part_host, k.a->part, (size_t)nvec * kKrylovBlocks * sizeof(double),
                                     cudaMemcpyDeviceToHost, k.s), "dots D2H");
  if (!rc) rc = cuda_status(cudaMemcpyAsync(k.a->ctl_host, k.a->ctl, sizeof(AdjCtl), cudaMemcpyDeviceToHost, k.s), "ctl D2H");
  if (!rc) rc = cuda_status(cudaStreamSynchronize(k.s), "dots");
  if (rc) return rc;
  if (k.a->ctl_host->err) k.err = k.a->ctl_host->err;
  for (int i = 0; i < nvec; ++i) {
    double t = 0.0;
    for (int b = 0; b < kKrylovBlocks; ++b) t += k.a->part_host[(size_t)i * kKrylovBlocks + b];
    hout[i] = t;
  }
  return UFE_OK;
}

int kry_axpy(Krylov &k, int nvec, const double *Vb, const double *coef, double *wv) {
  // A copy from pageable memory returns once the data is staged, so the caller may reuse
  // the coefficient array at once.
  int rc = cuda_status(cudaMemcpyAsync(k.a->hdev, coef, (size_t)nvec * sizeof(double), cudaMemcpyHostToDevice, k.s), "coef H2D");
  if (!rc) {
    k_krylov_axpy<<<(unsigned)((k.n + 255) / 256), 256, 0, k.s>>>(k.n, nvec, Vb, k.ld, k.a->hdev, wv);
    rc = cuda_status(cudaGetLastError(), "k_krylov_axpy");
  }
  return rc;
}

// Restarted GMRES(m) on (I - G) mu = S(0; g); classical Gram-Schmidt applied twice.
// Returns the relative residual of the preconditioned system in *rel; mu ends in a->mu.
int adj_gmres(Krylov &k, int m, double tol, int max_iter, double *rel, int *iters) {
  const unsigned gp = (unsigned)((k.nP + 255) / 256);
  // c = S(0; g)
  k_krylov_load<<<gp, 256, 0, k.s>>>(k.nP, nullptr, k.a->alpha, k.a->mu, k.a->s);
  int rc = cuda_status(cudaGetLastError(), "k_krylov_load");
  if (!rc) rc = kry_sweep(k, k.a->g);
  if (!rc) rc = cuda_status(cudaMemcpyAsync(k.c, k.a->mu, k.n * sizeof(double), cudaMemcpyDeviceToDevice, k.s), "copy c");
  if (!rc) rc = cuda_status(cudaMemsetAsync(k.x, 0, k.n * sizeof(double), k.s), "memset x");
  if (rc) return rc;
  double beta0 = 0.0;
  if ((rc = kry_dots(k, 1, k.c, k.c, &beta0))) return rc;
  beta0 = std::sqrt(beta0);
  *iters = 0;
  *rel = 0.0;
  if (beta0 == 0.0) {
    k_krylov_load<<<gp, 256, 0, k.s>>>(k.nP, nullptr, k.a->alpha, k.a->mu, k.a->s);
    return cuda_status(cudaGetLastError(), "k_krylov_load");
  }
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), gv(m + 1), hcol(m + 1), h2(m + 1), y(m);
  auto Hm = [&](int i, int j) -> double & { return H[(size_t)j * (m + 1) + i]; };
  int total = 0;
  double res = 1.0, cycle_start = 1.0;
  while (total < max_iter) {
    // r = c - A x (x = 0 on the first cycle)
    double *V0 = k.V;
    if (total == 0) {
      rc = cuda_status(cudaMemcpyAsync(V0, k.c, k.n * sizeof(double), cudaMemcpyDeviceToDevice, k.s), "copy r");
    } else {
      rc = kry_apply(k, k.x, k.w);
      if (!rc) {
        k_krylov_sub<<<(unsigned)((k.n + 255) / 256), 256, 0, k.s>>>(k.n, k.c, k.w, V0);
        rc = cuda_status(cudaGetLastError(), "k_krylov_sub");
      }
    }
    if (rc) return rc;
    double beta = 0.0;
    if ((rc = kry_dots(k, 1, V0, V0, &beta))) return rc;
    beta = std::sqrt(beta);
    if (beta <= tol * beta0) { res = beta / beta0; break; }
    k_krylov_scale<<<(unsigned)((k.n + 255) / 256), 256, 0, k.s>>>(k.n, V0, 1.0 / beta, V0);
    if ((rc = cuda_status(cudaGetLastError(), "k_krylov_scale"))) return rc;
    std::fill(gv.begin(), gv.end(), 0.0);
    gv[0] = beta;
    int j_end = 0;
    for (int j = 0; j < m && total < max_iter; ++j) {
      double *Vj = k.V + (size_t)j * k.ld;
      if ((rc = kry_apply(k, Vj, k.w))) return rc;
      if ((rc = kry_dots(k, j + 1, k.V, k.w, hcol.data()))) return rc;
      if ((rc = kry_axpy(k, j + 1, k.V, hcol.data(), k.w))) return rc;
      if ((rc = kry_dots(k, j + 1, k.V, k.w, h2.data()))) return rc;
      if ((rc = kry_axpy(k, j + 1, k.V, h2.data(), k.w))) return rc;
      for (int i = 0; i <= j; ++i) hcol[i] += h2[i];
      double nw = 0.0;
      if ((rc = kry_dots(k, 1, k.w, k.w, &nw))) return rc;
      nw = std::sqrt(nw);
      if (k.err) return k.err;
      for (int i = 0; i <= j; ++i) Hm(i, j) = hcol[i];
      Hm(j + 1, j) = nw;
      if (nw > 0.0) {
        k_krylov_scale<<<(unsigned)((k.n + 255) / 256), 256, 0, k.s>>>(k.n, k.w, 1.0 / nw, k.V + (size_t)(j + 1) * k.ld);
        if ((rc = cuda_status(cudaGetLastError(), "k_krylov_scale"))) return rc;
      }
      // Givens rotations: apply the previous ones to the new column, then make a new one
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * Hm(i, j) + sn[i] * Hm(i + 1, j);
        Hm(i + 1, j) = -sn[i] * Hm(i, j) + cs[i] * Hm(i + 1, j);
        Hm(i, j) = t;
      }
      const double r = std::hypot(Hm(j, j), Hm(j + 1, j));
      cs[j] = r > 0.0 ? Hm(j, j) / r : 1.0;
      sn[j] = r > 0.0 ? Hm(j + 1, j) / r : 0.0;
      Hm(j, j) = r;
      Hm(j + 1, j) = 0.0;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      ++total;
      j_end = j + 1;
      res = std::fabs(gv[j + 1]) / beta0;
      if (!std::isfinite(res)) return UFE_DIVERGED;
      if (res <= tol || nw == 0.0) break;
    }
    // x += V y, H y = g (upper triangular)
    for (int i = j_end - 1; i >= 0; --i) {
      double t = gv[i];
      for (int l = i + 1; l < j_end; ++l) t -= Hm(i, l) * y[l];
      y[i] = t / Hm(i, i);
    }
    for (int i = 0; i < j_end; ++i) y[i] = -y[i];
    if ((rc = kry_axpy(k, j_end, k.V, y.data(), k.x))) return rc;
    if (res <= tol) break;
    // a restart cycle that gains less than 5 % will not reach the tolerance: stop
    if (res > 0.95 * cycle_start) break;
    cycle_start = res;
  }
  *rel = res;
  *iters = total;
  // mu = x (and s consistent with it, for the gradient kernels that only read mu)
  k_krylov_load<<<gp, 256, 0, k.s>>>(k.nP, reinterpret_cast<const double2 *>(k.x), k.a->alpha, k.a->mu, k.a->s);
  return cuda_status(cudaGetLastError(), "k_krylov_load");
}

}  // namespace
}  // namespace ufe

extern "C" int ufe_ssa_vjp(ufe_mesh_h h, const ufe_params *p, const ufe_vjp_params *vp, const ufe_vjp_in *in,
                           const ufe_vjp_geom *geom, ufe_vjp_out *out, ufe_vjp_stats *stats) {
  if (!h || !p || !in || !out) { set_error("ufe_ssa_vjp: null argument"); return UFE_BAD_ARG; }
  SsaWork *w = h->ssa;
  if (!w || !w->uploaded) { set_error("ufe_ssa_vjp: no solve on this mesh handle"); return UFE_BAD_ARG; }
  if (w->zero) { set_error("ufe_ssa_vjp: the last solve took the zero-velocity early-out"); return UFE_BAD_ARG; }
  if (w->gl) { set_error("ufe_ssa_vjp: the grounding-line flux option is not differentiated"); return UFE_BAD_ARG; }
  if (p->sliding_law != UFE_SLIDING_LINEAR && p->sliding_law != UFE_SLIDING_COULOMB_REGULARISED) {
    set_error("ufe_ssa_vjp: unknown sliding law");
    return UFE_BAD_ARG;
  }
  const bool coulomb = p->sliding_law == UFE_SLIDING_COULOMB_REGULARISED;
  if (coulomb != (w->sliding_law == UFE_SLIDING_COULOMB_REGULARISED)) {
    set_error("ufe_ssa_vjp: the sliding law differs from the one of the last solve");
    return UFE_BAD_ARG;
  }
  if (!in->dJ_dU || !in->dJ_dV || !in->dJ_dUx_Ac || !in->dJ_dUy_Ac) { set_error("ufe_ssa_vjp: missing dJ/du"); return UFE_BAD_ARG; }
  if (out->dJ_dHi && (!geom || !geom->nC || !geom->C || !geom->Nx || !geom->Ny || !geom->Aci || !geom->Nx_Ac || !geom->Ny_Ac)) {
    set_error("ufe_ssa_vjp: dJ_dHi needs the Aa and Ac derivative stencils (ufe_vjp_geom)");
    return UFE_BAD_ARG;
  }
  int rc = ensure_adj(h);
  if (rc) return rc;
  AdjWork *a = h->adj;
  const DevMesh &m = h->m;
  cudaStream_t s = h->stream;
  const size_t nV = m.nV, nAc = m.nAc, nA = m.nA, nP = m.nP, ncm = m.ncm;
  // SOR: the error of a slowly contracting iteration is about its update / (1 - rate), so
  // the default stops only when updates reach 1e-13 of the state. GMRES: relative residual
  // of the sweep-preconditioned system.
  const bool gmres_default = !vp || vp->method == UFE_VJP_GMRES;
  const double tol = vp && vp->tol > 0 ? vp->tol : (gmres_default ? 1e-12 : 1e-13);
  const int max_sweeps = vp && vp->max_sweeps > 0 ? vp->max_sweeps : 2000000;
  const double omega = vp && vp->omega > 0 ? vp->omega : p->SSA_SOR_omega;
  double *st = a->stage;
  double *gU = st, *gV = st + nV, *gUx = st + 2 * nV, *gUy = gUx + nAc;
  double *o_lb = gUy + nAc, *o_hx = o_lb + nA, *o_hy = o_hx + nA, *o_H = o_hy + nA, *o_lU = o_H + nA, *o_lV = o_lU + nA;
  double *o_dHi = o_lV + nA, *o_phi = o_dHi + nV;
  std::memset(a->ctl_host, 0, sizeof(AdjCtl));
  rc = cuda_status(cudaEventRecord(a->ev0, s), "event");
  if (!rc) rc = h2d(gU, in->dJ_dU, nV, s);
  if (!rc) rc = h2d(gV, in->dJ_dV, nV, s);
  if (!rc) rc = h2d(gUx, in->dJ_dUx_Ac, nAc, s);
  if (!rc) rc = h2d(gUy, in->dJ_dUy_Ac, nAc, s);
  if (!rc) rc = cuda_status(cudaMemsetAsync(a->ctl, 0, sizeof(AdjCtl), s), "memset adj ctl");
  if (!rc) rc = cuda_status(cudaMemsetAsync(a->prog, 0, 32 * (size_t)m.n_patch * sizeof(unsigned int), s), "memset prog");
  const double *F = w->f;
  AdjSetup su;
  su.nP = (int)nP; su.nV = (int)nV; su.col = m.col; su.deg = m.deg; su.slice_e0 = m.slice_e0; su.slice_g = m.slice_g;
  su.orig_of_dev = m.orig_of_dev; su.nxy = m.nxy; su.h_nxy = m.h_nxy; su.h_cuv = m.h_cuv; su.sNxy = m.sNxy;
  su.Hi = F + F_HI * nP; su.Hb = F + F_HB * nP; su.SL = F + F_SL * nP; su.hx = F + F_HX * nP; su.hy = F + F_HY * nP;
  su.Af = F + F_AF * nP; su.beta = w->has_beta ? F + F_BETA * nP : nullptr;
  su.tau = F + F_TAU * nP; su.coulomb = coulomb ? 1 : 0;
  su.uq = std::pow(100.0, 0.30); su.expo = 0.5 * (0.30 - 1.0);   // u_threshold, q_plastic (727-779)
  su.beta_const = p->beta_sq; su.m_enh = p->m_enh_ssa; su.UV = w->UV;
  su.dJ_U = gU; su.dJ_V = gV; su.dJ_Ux = gUx; su.dJ_Uy = gUy;
  su.ee = a->ee; su.kh = a->kh; su.alpha = a->alpha; su.dinv = a->dinv; su.g = a->g; su.mu = a->mu;
  su.c3 = a->c3; su.s = a->s; su.eta = a->eta; su.fr = a->fr; su.inv_nb = a->inv_nb; su.K = a->K; su.omega = omega;
  const unsigned gb = (unsigned)((nP + 255) / 256);
  if (!rc) {
    k_adj_rows<<<gb, 256, 0, s>>>(su);
    rc = cuda_status(cudaGetLastError(), "k_adj_rows");
  }
  if (!rc) {
    k_adj_entries<<<gb, 256, 0, s>>>(su, a->cT, a->kT, m.cuv, a->ctl);
    rc = cuda_status(cudaGetLastError(), "k_adj_entries");
  }
  AdjArgs aa;
  aa.col = m.col; aa.deg = m.deg; aa.orig_of_dev = m.orig_of_dev; aa.slice_e0 = m.slice_e0; aa.slice_w = m.slice_w;
  aa.patch_slice = m.patch_slice; aa.patch_edge0 = m.patch_edge0; aa.sync_ptr = m.sync_ptr; aa.sync_list = m.sync_list;
  aa.prog = a->prog; aa.cT = a->cT; aa.kT = a->kT; aa.ee = a->ee; aa.c3 = a->c3; aa.kh = a->kh; aa.alpha = a->alpha;
  aa.dinv = a->dinv; aa.g = a->g; aa.mu = a->mu; aa.s = a->s; aa.ctl = a->ctl; aa.omega = omega; aa.tol = tol;
  aa.max_sweeps = max_sweeps; aa.timeout_ns = wait_timeout_ns();
  const bool krylov = !vp || vp->method == UFE_VJP_GMRES;
  int k_iters = 0, k_err = 0;
  double k_rel = 0.0;
  if (!rc && !krylov) {
    void *args[] = {(void *)&aa};
    rc = cuda_status(cudaLaunchCooperativeKernel((const void *)ssa_adjoint_sor, dim3(m.n_patch), dim3(kSsaBlock), args, 0, s),
                     "ssa_adjoint_sor");
  } else if (!rc) {
    const int restart = std::min(kMaxKrylovRestart, vp && vp->restart > 0 ? vp->restart : 100);
    const size_t n2 = 2 * nP;
    const size_t need = (size_t)(restart + 1) + 4;   // basis, w, x, c, zero rows
    if (a->kry_vectors < need) {
      if (a->kry) { cudaFree(a->kry); a->kry = nullptr; }
      rc = cuda_status(cudaMalloc(&a->kry, need * n2 * sizeof(double)), "krylov basis");
      if (!rc) a->kry_vectors = need;
    }
    if (!rc && !a->part) rc = cuda_status(cudaMalloc(&a->part, (size_t)(kMaxKrylovRestart + 1) * kKrylovBlocks * sizeof(double)), "krylov dots");
    if (!rc && !a->part_host) rc = cuda_status(cudaMallocHost(&a->part_host, (size_t)(kMaxKrylovRestart + 1) * kKrylovBlocks * sizeof(double)), "krylov dots host");
    if (!rc && !a->hdev) rc = cuda_status(cudaMalloc(&a->hdev, (size_t)(kMaxKrylovRestart + 1) * sizeof(double)), "krylov coefficients");
    if (!rc) {
      Krylov k;
      k.h = h; k.a = a; k.aa = aa; k.s = s; k.nP = (int)nP; k.n = (int)n2; k.ld = n2;
      k.V = a->kry; k.w = k.V + (size_t)(restart + 1) * n2; k.x = k.w + n2; k.c = k.x + n2;
      k.zero = reinterpret_cast<double2 *>(k.c + n2);
      k.sweeps_per_apply = vp && vp->sweeps_per_iteration > 0 ? vp->sweeps_per_iteration : 8;
      rc = cuda_status(cudaMemsetAsync(k.zero, 0, n2 * sizeof(double), s), "memset zero");
      const int max_iter = vp && vp->max_sweeps > 0 ? vp->max_sweeps : 50000;
      if (!rc) rc = adj_gmres(k, restart, tol, max_iter, &k_rel, &k_iters);
      k_iters = k.sweeps;
      k_err = k.err;
      if (rc == UFE_DIVERGED) { rc = UFE_OK; k_rel = HUGE_VAL; k_err = UFE_DIVERGED; }
    }
  }
  AdjGrad ag;
  ag.nP = (int)nP; ag.nV = (int)nV; ag.orig_of_dev = m.orig_of_dev; ag.deg = m.deg; ag.slice_g = m.slice_g;
  ag.UV = w->UV; ag.mu = a->mu; ag.eta = a->eta; ag.fr = a->fr; ag.Hi = F + F_HI * nP;
  ag.coulomb = coulomb ? 1 : 0; ag.phi = F + F_PHI * nP;
  ag.d_logbeta = o_lb; ag.s_hx = o_hx; ag.s_hy = o_hy; ag.s_H = o_H; ag.lam_U = o_lU; ag.lam_V = o_lV;
  ag.d_phi = o_phi;
  if (!rc) {
    k_adj_grad<<<gb, 256, 0, s>>>(ag);
    rc = cuda_status(cudaGetLastError(), "k_adj_grad");
  }
  if (!rc && out->dJ_dHi) {
    int *gi = a->geom_int;
    double *gd = a->geom_dbl;
    rc = cuda_status(cudaMemcpyAsync(gi, geom->nC, nV * sizeof(int), cudaMemcpyHostToDevice, s), "H2D geom");
    if (!rc) rc = cuda_status(cudaMemcpyAsync(gi + nV, geom->C, nV * ncm * sizeof(int), cudaMemcpyHostToDevice, s), "H2D geom");
    if (!rc) rc = cuda_status(cudaMemcpyAsync(gi + nV + nV * ncm, geom->Aci, 4 * nAc * sizeof(int), cudaMemcpyHostToDevice, s), "H2D geom");
    if (!rc) rc = h2d(gd, geom->Nx, nV * (ncm + 1), s);
    if (!rc) rc = h2d(gd + nV * (ncm + 1), geom->Ny, nV * (ncm + 1), s);
    if (!rc) rc = h2d(gd + 2 * nV * (ncm + 1), geom->Nx_Ac, 4 * nAc, s);
    if (!rc) rc = h2d(gd + 2 * nV * (ncm + 1) + 4 * nAc, geom->Ny_Ac, 4 * nAc, s);
    if (!rc) rc = cuda_status(cudaMemsetAsync(o_dHi, 0, nV * sizeof(double), s), "memset dHi");
    AdjGeom ge;
    ge.nV = (int)nV; ge.nAc = (int)nAc; ge.ncm = (int)ncm; ge.dev_of_orig = m.dev_of_orig;
    ge.Hi = F + F_HI * nP; ge.Hb = F + F_HB * nP; ge.SL = F + F_SL * nP;
    ge.s_hx = o_hx; ge.s_hy = o_hy; ge.s_H = o_H; ge.nC = gi; ge.C = gi + nV; ge.Aci = gi + nV + nV * ncm;
    ge.Nx = gd; ge.Ny = gd + nV * (ncm + 1); ge.Nx_Ac = gd + 2 * nV * (ncm + 1); ge.Ny_Ac = ge.Nx_Ac + 4 * nAc;
    ge.dHi = o_dHi;
    if (!rc) {
      k_adj_geom<<<(unsigned)((nA + 255) / 256), 256, 0, s>>>(ge);
      rc = cuda_status(cudaGetLastError(), "k_adj_geom");
    }
  }
  if (!rc) rc = cuda_status(cudaEventRecord(a->ev1, s), "event");
  if (!rc) rc = cuda_status(cudaMemcpyAsync(a->ctl_host, a->ctl, sizeof(AdjCtl), cudaMemcpyDeviceToHost, s), "ctl D2H");
  if (!rc) rc = d2h(out->dJ_dlogbeta_sq_AaAc, o_lb, nA, s);
  if (!rc) rc = d2h(out->dJ_dhx_AaAc, o_hx, nA, s);
  if (!rc) rc = d2h(out->dJ_dhy_AaAc, o_hy, nA, s);
  if (!rc) rc = d2h(out->dJ_dHi_AaAc, o_H, nA, s);
  if (!rc) rc = d2h(out->lambda_U_AaAc, o_lU, nA, s);
  if (!rc) rc = d2h(out->lambda_V_AaAc, o_lV, nA, s);
  if (!rc && out->dJ_dHi) rc = d2h(out->dJ_dHi, o_dHi, nV, s);
  if (!rc && coulomb) rc = d2h(out->dJ_dphi_fric_AaAc, o_phi, nA, s);
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s), "ssa vjp");
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a->ev0, a->ev1);
  const AdjCtl &c = *a->ctl_host;
  int status = c.status;
  if (krylov) {
    status = k_err ? k_err : (k_rel <= tol ? UFE_OK : UFE_NOT_CONVERGED);
    if (status == UFE_DIVERGED) set_error("ufe_ssa_vjp: GMRES produced a non-finite residual");
    else if (status == UFE_NOT_CONVERGED) set_error("ufe_ssa_vjp: the GMRES iteration limit was reached before the tolerance");
    a->ctl_host->sweeps = k_iters;
    a->ctl_host->last_rel = k_rel;
  }
  if (status == UFE_DIVERGED) set_error("ufe_ssa_vjp: the transposed SOR diverged (lower the relaxation factor)");
  else if (status == UFE_NOT_CONVERGED) set_error("ufe_ssa_vjp: max_sweeps reached before the tolerance");
  if (c.err) { status = c.err; set_error("ufe_ssa_vjp: a device-side bounded wait timed out"); }
  else if (c.not_found) { status = UFE_BAD_MESH; set_error("ufe_ssa_vjp: the AaAc neighbour relation is not symmetric"); }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->status = status;
    stats->sweeps = c.sweeps;
    stats->last_rel_update = c.last_rel;
    stats->device_ms = ms;
  }
  return status;
}

#if UFE_PHASE_TIMERS
// Profiling build only (not part of the C-ABI header): the per-phase SM-cycle totals of the
// persistent solver summed over CTAs since the last reset, in PhaseTimer order; `reset`
// zeroes them after the read.
extern "C" int ufe_debug_phase_cycles(unsigned long long *out, int n, int reset) {
  // out: kTmCount totals, then (if n allows) kTmCount per CTA for up to kTmMaxCta CTAs
  if (!out || n < (int)kTmCount) { set_error("ufe_debug_phase_cycles: need kTmCount slots"); return UFE_BAD_ARG; }
  int rc = cuda_status(cudaDeviceSynchronize(), "ufe_debug_phase_cycles");
  if (!rc) rc = cuda_status(cudaMemcpyFromSymbol(out, g_phase_cycles, sizeof(unsigned long long) * kTmCount),
                            "read phase timers");
  const int per = std::min(kTmMaxCta * kTmCount, n - (int)kTmCount);
  if (!rc && per > 0)
    rc = cuda_status(cudaMemcpyFromSymbol(out + kTmCount, g_phase_cycles_cta, sizeof(unsigned long long) * per),
                     "read phase timers per CTA");
  if (!rc && reset) {
    static const unsigned long long zeros[kTmCount] = {};
    rc = cuda_status(cudaMemcpyToSymbol(g_phase_cycles, zeros, sizeof(zeros)), "reset phase timers");
    std::vector<unsigned long long> z((size_t)kTmMaxCta * kTmCount, 0ull);
    if (!rc) rc = cuda_status(cudaMemcpyToSymbol(g_phase_cycles_cta, z.data(), z.size() * sizeof(unsigned long long)),
                              "reset phase timers per CTA");
  }
  return rc ? rc : (int)kTmCount;
}
#endif
