// FP64 path: the reference's arithmetic, operation for operation, on the GPU.
//
// This translation unit is compiled with --fmad=false, so every expression
// below rounds exactly like the reference built with -ffp-contract=off.  Per
// particle the neighbour sums run in the reference's order (cell stencil
// order, ascending members; Verlet list order), so cell ids, member lists and
// Verlet lists are bit-identical to the reference's and floating-point
// results differ only by the last bits of the device sin/cos/atan2/hypot and
// by the all-pairs sum order.  Layout: AoS double[n*s], as the reference.
//
// Reference: DynamicalSystems/ParticleSystemFirstOrder.cpp, ParticleSystemFirstOrderPtr.cpp,
// ParticleSystemSecondOrder.cpp, BoundaryConfiguration/PeriodicBoundaryConditions.cpp,
// Steppers/*.
#include <algorithm>
#include <cstring>

#include "spss_internal.cuh"

namespace spss
{

struct F64Path
{
  DeviceArray<double> state, rk, k[4], td, det, caf, nat_freq, partials, scratch_state, scratch_kprev,
      scratch_knext;
  DeviceArray<int> cell_of;
  DeviceArray<float2> posf;  // stage positions wrapped into the box, float (all-pairs range pre-test)
  DeviceArray<double2> csphi;  // cos and sin of the stage phase (all pairs: written with the stage)
  // the other stage buffers of an all-pairs RK4 step, whose pair kernels
  // write the next stage's state while they read this one's
  DeviceArray<double> rk2;
  DeviceArray<float2> posf2;
  DeviceArray<double2> csphi2;
  Binner binner;
  int cells_nc = 0;  // cells per side of the last build (0: none)
  DeviceArray<int> vl_count, vl_off, vl_ent;
  long vl_total = 0;
  int vl_built = 0;
  DeviceArray<unsigned long long> max2;
  unsigned long long *h_max2 = nullptr;  // pinned
  // one RK4 step captured as a CUDA graph (f64_steps), for the dt and
  // higher-order flag it was captured with
  cudaGraph_t rk4_graph = nullptr;
  cudaGraphExec_t rk4_exec = nullptr;
  double rk4_dt = 0.0;
  int rk4_higher_order = -1;
  unsigned long long rk4_launches = 0;  // kernels in the captured step
};

struct K64
{
  int model, flavor, n, s;
  double v0, xi, xi_r, xi_phi, sigma, alpha, rho2, rmax2, ca, sa;
  int higher_order;
  float rho_excl;  // a pair whose float minimum-image distance bound exceeds this is out of range
};

// Margin of the all-pairs range pre-test, in box units: covers the float
// rounding of the wrapped positions and of the bound (a few 1e-8) and the
// FP64 wrap of positions up to 1e4 boxes away (1e-12), many times over.
constexpr float kPretestMargin = 2e-5f;

static K64 make_k64(const spss_ctx *ctx)
{
  K64 k;
  const spss_params &p = ctx->p;
  k.model = p.model;
  k.flavor = p.flavor;
  k.n = p.n;
  k.s = ctx->s;
  k.v0 = p.v0;
  k.xi = p.xi;
  k.xi_r = p.xi_r;
  k.xi_phi = p.xi_phi;
  k.sigma = p.sigma;
  k.alpha = p.alpha;
  k.rho2 = p.rho * p.rho;
  k.rmax2 = ctx->r_max * ctx->r_max;
  k.ca = std::cos(p.alpha);  // host libm, as the reference's constructor
  k.sa = std::sin(p.alpha);
  k.higher_order = ctx->higher_order;
  k.rho_excl = (float) (p.rho + 2.0 * kPretestMargin);
  return k;
}

// ------------------------------------------------------------ PBC helpers

// ClassAEffectiveParticleDistance, unit box (PeriodicBoundaryConditions.cpp:26-38).
__device__ __forceinline__ double class_a(double d)
{
  return d - (double) (int) (d * 2.0 * 1.0) * 1.0;
}

// ClassCEffectiveParticleDistanceUnsigned, unit box (PeriodicBoundaryConditions.cpp:107-119).
__device__ __forceinline__ double class_c(double d)
{
  d = fabs(d);
  return d - (double) (int) (d * 1.0 + 0.5) * 1.0;
}

// ApplyPeriodicBoundaryConditions(x, y, ...) (PeriodicBoundaryConditions.cpp:121-125).
__device__ __forceinline__ double wrap1(double x)
{
  return x - floor(x * 1.0) * 1.0;
}

// Second-order classes wrap only positions that left the box (ParticleSystemSecondOrder.cpp:323-326).
__device__ __forceinline__ void wrap_if_outside(double &x, double &y)
{
  if (x < 0.0 || x >= 1.0 || y < 0.0 || y >= 1.0)
  {
    x = wrap1(x);
    y = wrap1(y);
  }
}

// int(x / x_size * num_subcells) (ParticleSystemFirstOrder.cpp:277-279); the
// reference's out-of-range result for a coordinate that rounds to the box
// edge is clamped to the last cell.
__device__ __forceinline__ int cell_coord(double x, int nc)
{
  int c = (int) (x / 1.0 * nc);
  return c >= nc ? nc - 1 : (c < 0 ? 0 : c);
}

// AdjustNeighboringCellToPeriodicBoundaries (ParticleSystemFirstOrder.cpp:651-668).
__device__ __forceinline__ int adjust_cell(int c, int nc)
{
  return c < 0 ? nc - 1 : (c >= nc ? 0 : c);
}

// neighboring_cells_ (ParticleSystemFirstOrder.cpp:47-52).
__constant__ int c_stencil[9][2] = {{-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {0, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1}};

__device__ __forceinline__ void pos_for_cells(const K64 &k, const double *rk, int i, double &x, double &y)
{
  x = rk[(long) k.s * i];
  y = rk[(long) k.s * i + 1];
  if (k.model == 1)
  {
    x = wrap1(x);
    y = wrap1(y);
  } else
  {
    wrap_if_outside(x, y);
  }
}

// dr^2 of one candidate pair as the given class computes it.  The
// second-order all-pairs routine uses x_j as is; its linked-list routine
// wraps x_j if it left the box (ParticleSystemSecondOrder.cpp:380-385).
template<bool WRAP_J>
__device__ __forceinline__ double pair_dr2(const K64 &k, double x_i, double y_i, double x_j, double y_j)
{
  double dx, dy;
  if (k.model == 1)
  {
    dx = class_c(x_j - x_i);
    dy = class_c(y_j - y_i);
  } else
  {
    if (WRAP_J) wrap_if_outside(x_j, y_j);
    dx = class_a(x_j - x_i);
    dy = class_a(y_j - y_i);
  }
  return dx * dx + dy * dy;
}

struct Sums
{
  double af, card, caf;
};

// Pair terms: first order ParticleSystemFirstOrderPtr.cpp:404-415; second
// order ParticleSystemSecondOrder.cpp:160-161 (its complementary force is the
// first-order term in the second-order sin(phi_j - phi_i - alpha) convention).
__device__ __forceinline__ void add_pair(const K64 &k, Sums &a, double phi_i, double omega_i, double phi_j,
                                         double omega_j)
{
  if (k.model == 1)
  {
    a.af += sin(phi_j - phi_i) * k.ca - cos(phi_j - phi_i) * k.sa;
    a.card += 1.0;
    if (k.higher_order) a.caf += (omega_j - omega_i) * (cos(phi_j - phi_i) * k.ca + sin(phi_j - phi_i) * k.sa);
  } else
  {
    a.af += sin(phi_j - phi_i - k.alpha);
    a.card += 1.0;
    if (k.higher_order) a.caf += (omega_j - omega_i) * cos(phi_j - phi_i - k.alpha);
  }
}

// Output of one particle (ParticleSystemFirstOrder.cpp:220-226, ParticleSystemSecondOrder.cpp:166-175);
// the torque component is left untouched when the particle has no neighbour.
// `cs`: cos and sin of the particle's phase computed beforehand (the same
// functions of the same value), or null.
__device__ __forceinline__ void write_k(const K64 &k, int i, const double *st, Sums a, double *k_next, double *caf,
                                        const double2 *cs = nullptr)
{
  const long ii = (long) k.s * i;
  if (k.model == 1)
  {
    const double phi_i = st[2], omega_i = st[3];
    k_next[ii] = k.v0 * (cs ? cs->x : cos(phi_i));
    k_next[ii + 1] = k.v0 * (cs ? cs->y : sin(phi_i));
    k_next[ii + 2] = omega_i;
    if (a.card != 0.0)
    {
      k_next[ii + 3] = -k.xi * omega_i + k.sigma * a.af / a.card;
      if (k.higher_order) a.caf *= k.sigma / a.card;
    }
  } else
  {
    const double v_x_i = st[2], v_y_i = st[3], phi_i = st[4], omega_i = st[5];
    k_next[ii] = v_x_i;
    k_next[ii + 1] = v_y_i;
    k_next[ii + 2] = -k.xi_r * v_x_i + k.v0 * (cs ? cs->x : cos(phi_i));
    k_next[ii + 3] = -k.xi_r * v_y_i + k.v0 * (cs ? cs->y : sin(phi_i));
    k_next[ii + 4] = omega_i;
    if (a.card != 0.0)
    {
      k_next[ii + 5] = -k.xi_phi * omega_i + k.sigma * a.af / a.card;
      if (k.higher_order) a.caf *= k.sigma / a.card;
    }
  }
  if (k.higher_order) caf[i] = a.caf;
}

// ------------------------------------------------------------ kernels

// rk_system_state = system_state + k_coef * dt * k_prev (ParticleSystemFirstOrder.cpp:175-184).
__global__ void f64_stage_kernel(const double *__restrict__ st, const double *__restrict__ kp,
                                 double *__restrict__ rk, long len, double k_coef, double dt)
{
  const long q = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (q < len) rk[q] = st[q] + k_coef * dt * kp[q];
}

__global__ void f64_cell_kernel(K64 k, const double *__restrict__ rk, int nc, int *__restrict__ cell_of)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  double x, y;
  pos_for_cells(k, rk, i, x, y);
  cell_of[i] = cell_coord(y, nc) * nc + cell_coord(x, nc);
}

// The stage state of one particle per thread (the same expression as
// f64_stage_kernel, element by element), its position wrapped into the
// unit box as floats, for the all-pairs range pre-test, and the cos and sin
// of its phase for its own derivative (one thread per particle here, where
// the pair kernel would spend a whole warp's FP64 pipe time on one lane).
__global__ void f64_stage_posf_kernel(K64 k, const double *__restrict__ st, const double *__restrict__ kp,
                                      double *__restrict__ rk, float2 *__restrict__ posf,
                                      double2 *__restrict__ csphi, double k_coef, double dt)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  const long ii = (long) k.s * i;
  for (int q = 0; q < k.s; ++q) rk[ii + q] = st[ii + q] + k_coef * dt * kp[ii + q];
  const double x = rk[ii], y = rk[ii + 1];
  posf[i] = make_float2((float) (x - floor(x)), (float) (y - floor(y)));
  const double phi = rk[ii + (k.model == 1 ? 2 : 4)];
  csphi[i] = make_double2(cos(phi), sin(phi));
}

// A lower bound of the minimum-image distance of two particles from their
// float wrapped positions (exact minimum image of the wrapped coordinates,
// less the margin): every periodic image the reference's distance functions
// may pick is at least this far, so a pair whose bound exceeds rho is out of
// range for the FP64 test as well.
__device__ __forceinline__ bool pretest_out(const K64 &k, float2 a, float2 b)
{
  float dx = fabsf(b.x - a.x), dy = fabsf(b.y - a.y);
  dx = fmaxf(fminf(dx, 1.0f - dx) - kPretestMargin, 0.0f);
  dy = fmaxf(fminf(dy, 1.0f - dy) - kPretestMargin, 0.0f);
  return dx > k.rho_excl || dy > k.rho_excl || dx * dx + dy * dy > k.rho_excl * k.rho_excl;
}

// The next RK4 stage, written by the pair kernel of this one (null rk: none):
// rk = x + coef * dt * k_next, its wrapped float position and the cos and sin
// of its phase, the expressions of f64_stage_posf_kernel.
struct NextStage
{
  const double *x;
  double coef, dt;
  double *rk;
  float2 *posf;
  double2 *csphi;
};

// All pairs (ParticleSystemFirstOrder.cpp:162-228, ParticleSystemFirstOrderPtr.cpp:225-316,
// ParticleSystemSecondOrder.cpp:116-177): one warp per particle, lanes stride
// over j, partial sums combined by a fixed shuffle tree.  A float pre-test
// on the wrapped positions excludes the pairs that are certainly out of
// range; every other pair is decided by the reference's FP64 expression, so
// the neighbour sets are the FP64 ones.
__global__ void f64_allpairs_kernel(K64 k, const double *__restrict__ rk, const float2 *__restrict__ posf,
                                    const double2 *__restrict__ csphi, double *__restrict__ k_next,
                                    double *__restrict__ caf, NextStage next)
{
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= k.n) return;
  const int i = warp;
  const int ip = k.model == 1 ? 2 : 4;
  const double *st = rk + (long) k.s * i;
  double x_i = st[0], y_i = st[1];
  const double phi_i = st[ip], omega_i = st[ip + 1];
  if (k.model == 1 && k.flavor == 1)
  {
    x_i = wrap1(x_i);
    y_i = wrap1(y_i);
  }
  const float2 pi = posf[i];
  Sums a{0.0, 0.0, 0.0};
  // the lane's candidates j = lane, lane + 32, ... in that order; the float
  // positions of four of them are loaded together.  The pair terms (FP64 sin
  // and cos, a warp's full FP64 pipe time whatever the lanes) wait until the
  // scan is over, so the few neighbours of a particle, found by different
  // lanes in different iterations, are summed in one pass; each lane still
  // adds its own neighbours in ascending j, so the sums are unchanged.
  int pend[4], np = 0;
  for (int j0 = lane; j0 < k.n; j0 += 128)
  {
    float2 pj[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) pj[u] = j0 + 32 * u < k.n ? posf[j0 + 32 * u] : pi;
#pragma unroll
    for (int u = 0; u < 4; ++u)
    {
      const int j = j0 + 32 * u;
      if (j >= k.n || j == i || pretest_out(k, pi, pj[u])) continue;
      const double *sj = rk + (long) k.s * j;
      if (pair_dr2<false>(k, x_i, y_i, sj[0], sj[1]) <= k.rho2)
      {
        if (np == 4)
        {
          for (int t = 0; t < 4; ++t)
          {
            const double *sp = rk + (long) k.s * pend[t];
            add_pair(k, a, phi_i, omega_i, sp[ip], sp[ip + 1]);
          }
          np = 0;
        }
        pend[np++] = j;
      }
    }
  }
  for (int t = 0; t < np; ++t)
  {
    const double *sp = rk + (long) k.s * pend[t];
    add_pair(k, a, phi_i, omega_i, sp[ip], sp[ip + 1]);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
  {
    a.af += __shfl_xor_sync(0xffffffffu, a.af, off);
    a.card += __shfl_xor_sync(0xffffffffu, a.card, off);
    a.caf += __shfl_xor_sync(0xffffffffu, a.caf, off);
  }
  if (lane != 0) return;
  write_k(k, i, st, a, k_next, caf, csphi + i);
  if (next.rk)
  {
    // this particle's derivative is complete (an entry write_k left untouched
    // keeps the value it had, as the stage kernel would read it)
    const long ii = (long) k.s * i;
    for (int q = 0; q < k.s; ++q) next.rk[ii + q] = next.x[ii + q] + next.coef * next.dt * k_next[ii + q];
    const double x = next.rk[ii], y = next.rk[ii + 1];
    next.posf[i] = make_float2((float) (x - floor(x)), (float) (y - floor(y)));
    const double phi = next.rk[ii + (k.model == 1 ? 2 : 4)];
    next.csphi[i] = make_double2(cos(phi), sin(phi));
  }
}

// Linked list (ParticleSystemFirstOrder.cpp:231-353, ParticleSystemSecondOrder.cpp:276-409).
__global__ void f64_linked_list_kernel(K64 k, const double *__restrict__ rk, int nc, const int *__restrict__ off,
                                       const int *__restrict__ mem, double *__restrict__ k_next,
                                       double *__restrict__ caf)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  const int ip = k.model == 1 ? 2 : 4;
  const double *st = rk + (long) k.s * i;
  double x_i, y_i;
  pos_for_cells(k, rk, i, x_i, y_i);
  const double phi_i = st[ip], omega_i = st[ip + 1];
  const int cx = cell_coord(x_i, nc), cy = cell_coord(y_i, nc);
  Sums a{0.0, 0.0, 0.0};
  for (int c = 0; c < 9; ++c)
  {
    const int jc = adjust_cell(cy + c_stencil[c][1], nc) * nc + adjust_cell(cx + c_stencil[c][0], nc);
    for (int m = off[jc]; m < off[jc + 1]; ++m)
    {
      const int j = mem[m];
      if (j == i) continue;
      const double *sj = rk + (long) k.s * j;
      if (pair_dr2<true>(k, x_i, y_i, sj[0], sj[1]) <= k.rho2) add_pair(k, a, phi_i, omega_i, sj[ip], sj[ip + 1]);
    }
  }
  write_k(k, i, st, a, k_next, caf);
}

// Verlet list from the cell list (ParticleSystemFirstOrder.cpp:536-589): first
// pass counts, second pass fills in the reference's push_back order.
template<bool FILL>
__global__ void f64_verlet_cells_kernel(K64 k, const double *__restrict__ rk, int nc, const int *__restrict__ off,
                                        const int *__restrict__ mem, int *__restrict__ count,
                                        const int *__restrict__ vl_off, int *__restrict__ vl_ent)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  double x_i, y_i;
  pos_for_cells(k, rk, i, x_i, y_i);
  const int cx = cell_coord(x_i, nc), cy = cell_coord(y_i, nc);
  int cnt = 0;
  int base = FILL ? vl_off[i] : 0;
  for (int c = 0; c < 9; ++c)
  {
    const int jc = adjust_cell(cy + c_stencil[c][1], nc) * nc + adjust_cell(cx + c_stencil[c][0], nc);
    for (int m = off[jc]; m < off[jc + 1]; ++m)
    {
      const int j = mem[m];
      if (j == i) continue;
      const double *sj = rk + (long) k.s * j;
      if (pair_dr2<true>(k, x_i, y_i, sj[0], sj[1]) <= k.rmax2)
      {
        if (FILL) vl_ent[base + cnt] = j;
        ++cnt;
      }
    }
  }
  if (!FILL) count[i] = cnt;
}

// Verlet list by an O(N^2) scan (ParticleSystemFirstOrder.cpp:376-422).
template<bool FILL>
__global__ void f64_verlet_all_kernel(K64 k, const double *__restrict__ rk, int *__restrict__ count,
                                      const int *__restrict__ vl_off, int *__restrict__ vl_ent)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  double x_i = rk[(long) k.s * i], y_i = rk[(long) k.s * i + 1];
  if (k.model == 2) wrap_if_outside(x_i, y_i);
  int cnt = 0;
  const int base = FILL ? vl_off[i] : 0;
  for (int j = 0; j < k.n; ++j)
  {
    if (j == i) continue;
    if (pair_dr2<true>(k, x_i, y_i, rk[(long) k.s * j], rk[(long) k.s * j + 1]) <= k.rmax2)
    {
      if (FILL) vl_ent[base + cnt] = j;
      ++cnt;
    }
  }
  if (!FILL) count[i] = cnt;
}

// Pair loop over the Verlet list (ParticleSystemFirstOrder.cpp:594-648, ParticleSystemFirstOrderPtr.cpp:861-930).
__global__ void f64_verlet_pairs_kernel(K64 k, const double *__restrict__ rk, const int *__restrict__ vl_off,
                                        const int *__restrict__ vl_ent, double *__restrict__ k_next,
                                        double *__restrict__ caf)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  const int ip = k.model == 1 ? 2 : 4;
  const double *st = rk + (long) k.s * i;
  double x_i = st[0], y_i = st[1];
  if (k.model == 2) wrap_if_outside(x_i, y_i);
  const double phi_i = st[ip], omega_i = st[ip + 1];
  Sums a{0.0, 0.0, 0.0};
  for (int m = vl_off[i]; m < vl_off[i + 1]; ++m)
  {
    const int j = vl_ent[m];
    if (j == i) continue;
    const double *sj = rk + (long) k.s * j;
    if (pair_dr2<true>(k, x_i, y_i, sj[0], sj[1]) <= k.rho2) add_pair(k, a, phi_i, omega_i, sj[ip], sj[ip + 1]);
  }
  write_k(k, i, st, a, k_next, caf);
}

// Global polar order field, first order (ParticleSystemFirstOrder.cpp:122-159,
// ParticleSystemFirstOrderPtr.cpp:155-223): block partial sums, then one block
// adds them in a fixed order.
__global__ void f64_field_partials_kernel(K64 k, const double *__restrict__ rk, double *__restrict__ partials)
{
  __shared__ double sh[4][256];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k.n; i += gridDim.x * blockDim.x)
  {
    const double phi = rk[(long) k.s * i + 2], om = rk[(long) k.s * i + 3];
    const double c = cos(phi), s = sin(phi);
    acc[0] += c;
    acc[1] += s;
    acc[2] += om * c;
    acc[3] += om * s;
  }
  for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1)
  {
    if ((int) threadIdx.x < w)
      for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; ++q) partials[4 * blockIdx.x + q] = sh[q][0];
}

__global__ void f64_field_apply_kernel(K64 k, const double *__restrict__ rk, const double *__restrict__ partials,
                                       int nparts, const double *__restrict__ nat_freq, double *__restrict__ k_next,
                                       double *__restrict__ caf)
{
  double tot[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = 0; b < nparts; ++b)
    for (int q = 0; q < 4; ++q) tot[q] += partials[4 * b + q];
  const double pre = tot[0] / k.n, pim = tot[1] / k.n, wre = tot[2] / k.n, wim = tot[3] / k.n;
  const double pabs = hypot(pre, pim), parg = atan2(pim, pre);
  const double wabs = hypot(wre, wim), warg = atan2(wim, wre);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k.n) return;
  const long ii = (long) k.s * i;
  const double phi_i = rk[ii + 2], omega_i = rk[ii + 3];
  k_next[ii] = k.v0 * cos(phi_i);
  k_next[ii + 1] = k.v0 * sin(phi_i);
  k_next[ii + 2] = omega_i;
  k_next[ii + 3] = -k.xi * omega_i + nat_freq[i]
      + k.sigma * pabs * (sin(parg - phi_i) * k.ca - cos(parg - phi_i) * k.sa);
  if (k.flavor == 1 && k.higher_order)
  {
    // the last sine uses arg(weighted field) as ParticleSystemFirstOrderPtr.cpp:219 does
    caf[i] = k.sigma * (wabs * (cos(warg - phi_i) * k.ca + sin(warg - phi_i) * k.sa)
        - omega_i * pabs * (cos(parg - phi_i) * k.ca + sin(warg - phi_i) * k.sa));
  }
}

// ------------------------------------------------------------ steppers

// RK4 combine (RungeKutta4Stepper.cpp:56-59): td = (k1 + 2 k2 + 2 k3 + k4) dt / 6; x += td.
__global__ void f64_rk4_combine_kernel(double *__restrict__ x, const double *__restrict__ k1,
                                       const double *__restrict__ k2, const double *__restrict__ k3,
                                       const double *__restrict__ k4, double *__restrict__ td, long len, double dt)
{
  const long q = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= len) return;
  const double d = (k1[q] + 2.0 * k2[q] + 2.0 * k3[q] + k4[q]) * dt / 6.0;
  td[q] = d;
  x[q] += d;
}

// Second-order stochastic Euler (StochasticEulerStepper.hpp:33-51 with
// ParticleSystemSecondOrder::AddNoise, ParticleSystemSecondOrder.cpp:439-451).
__global__ void f64_se2_kernel(double *__restrict__ x, const double *__restrict__ det, double *__restrict__ td,
                               int n, double dt, double sqrt_dt, double intensity_r, double intensity_phi,
                               NoiseKey nk)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double z[4];
  normals4_f64(nk, (uint32_t) i, 0, z);
  double stoch[6] = {0.0, 0.0, intensity_r * z[0], intensity_r * z[1], 0.0, intensity_phi * z[2]};
  const long ii = 6L * i;
  for (int s = 0; s < 6; ++s)
  {
    const double d = dt * det[ii + s] + sqrt_dt * stoch[s];
    td[ii + s] = d;
    x[ii + s] += d;
  }
}

// First-order stochastic Euler (StochasticEulerStepperPtr.hpp:40-73).
__global__ void f64_se1_kernel(double *__restrict__ x, const double *__restrict__ d, double *__restrict__ td, int n,
                               double dt, double sqrt_dt, double intensity_phi, NoiseKey nk)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double z[4];
  normals4_f64(nk, (uint32_t) i, 0, z);
  const double delta_W_phi = sqrt_dt * z[0];
  const long ii = 4L * i;
  td[ii] = d[ii] * dt;
  td[ii + 1] = d[ii + 1] * dt;
  td[ii + 2] = d[ii + 2] * dt;
  td[ii + 3] = d[ii + 3] * dt + intensity_phi * delta_W_phi;
  for (int s = 0; s < 4; ++s) x[ii + s] += td[ii + s];
}

// First-order strong order 1.5 Taylor scheme (StochasticRungeKuttaStepperPtr.hpp:40-76).
__global__ void f64_srk1_kernel(double *__restrict__ x, const double *__restrict__ d, const double *__restrict__ caf,
                                double *__restrict__ td, int n, double dt, double sqrt_dt, double dt15,
                                double inv_sqrt3, double sqrt_2noise, double friction, NoiseKey nk)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double z[4];
  normals4_f64(nk, (uint32_t) i, 0, z);
  const double U_1 = z[0], U_2 = z[1];
  const double delta_W_i = U_1 * sqrt_dt;
  const double delta_Z_i = 0.5 * dt15 * (U_1 + inv_sqrt3 * U_2);
  const long ii = 4L * i;
  td[ii] = d[ii] * dt - 0.5 * d[ii + 2] * d[ii + 1] * dt * dt;
  td[ii + 1] = d[ii + 1] * dt + 0.5 * d[ii + 2] * d[ii] * dt * dt;
  td[ii + 2] = d[ii + 2] * dt + 0.5 * d[ii + 3] * dt * dt + sqrt_2noise * delta_Z_i;
  td[ii + 3] = d[ii + 3] * dt + 0.5 * (caf[i] - friction * d[ii + 3]) * dt * dt
      + sqrt_2noise * (delta_W_i - friction * delta_Z_i);
  for (int s = 0; s < 4; ++s) x[ii + s] += td[ii + s];
}

// Second-order strong order 1.5 Taylor scheme (no reference code): the
// first-order scheme's construction applied to the second-order drift with
// additive noise on v_x, v_y (b_r) and omega (b_phi); see spss_oracle.c.
__global__ void f64_srk2_kernel(double *__restrict__ x, const double *__restrict__ d, const double *__restrict__ caf,
                                double *__restrict__ td, int n, double dt, double sqdt, double dt15, double inv_sqrt3,
                                double b_r, double b_phi, double xi_r, double xi_phi, double v0, NoiseKey nk)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double u[8];
  normals4_f64(nk, (uint32_t) i, 0, u);
  normals4_f64(nk, (uint32_t) i, 1, u + 4);
  const double dWx = u[0] * sqdt, dZx = 0.5 * dt15 * (u[0] + inv_sqrt3 * u[1]);
  const double dWy = u[2] * sqdt, dZy = 0.5 * dt15 * (u[2] + inv_sqrt3 * u[3]);
  const double dWw = u[4] * sqdt, dZw = 0.5 * dt15 * (u[4] + inv_sqrt3 * u[5]);
  const long ii = 6L * i;
  const double phi = x[ii + 4];
  const double cphi = cos(phi), sphi = sin(phi);
  td[ii] = d[ii] * dt + 0.5 * d[ii + 2] * dt * dt + b_r * dZx;
  td[ii + 1] = d[ii + 1] * dt + 0.5 * d[ii + 3] * dt * dt + b_r * dZy;
  td[ii + 2] = d[ii + 2] * dt + 0.5 * (-xi_r * d[ii + 2] - v0 * sphi * d[ii + 4]) * dt * dt + b_r * (dWx - xi_r * dZx);
  td[ii + 3] = d[ii + 3] * dt + 0.5 * (-xi_r * d[ii + 3] + v0 * cphi * d[ii + 4]) * dt * dt + b_r * (dWy - xi_r * dZy);
  td[ii + 4] = d[ii + 4] * dt + 0.5 * d[ii + 5] * dt * dt + b_phi * dZw;
  td[ii + 5] = d[ii + 5] * dt + 0.5 * (caf[i] - xi_phi * d[ii + 5]) * dt * dt + b_phi * (dWw - xi_phi * dZw);
  for (int s = 0; s < 6; ++s) x[ii + s] += td[ii + s];
}

// max_i (dx^2 + dy^2) of a displacement array (ParticleSystemFirstOrder.cpp:672-684);
// non-negative doubles order like their bit patterns.
__global__ void f64_max2_kernel(const double *__restrict__ td, int n, int s, unsigned long long *__restrict__ out)
{
  __shared__ double sh[256];
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    const double dx = td[(long) s * i], dy = td[(long) s * i + 1];
    const double d2 = dx * dx + dy * dy;
    if (m < d2) m = d2;
  }
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1)
  {
    if ((int) threadIdx.x < w && sh[threadIdx.x] < sh[threadIdx.x + w]) sh[threadIdx.x] = sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(out, (unsigned long long) __double_as_longlong(sh[0]));
}

__global__ void f64_noise_kernel(double *__restrict__ out, int n, int per, NoiseKey nk)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double u[8];
  normals4_f64(nk, (uint32_t) i, 0, u);
  if (per > 4) normals4_f64(nk, (uint32_t) i, 1, u + 4);
  for (int d = 0; d < per; ++d) out[(long) per * i + d] = u[d];
}

// ApplyPeriodicBoundaryConditions(system_state) (PeriodicBoundaryConditions.cpp:127-135).
__global__ void f64_pbc_kernel(double *__restrict__ x, int n, int s)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long ii = (long) s * i;
  x[ii] -= floor(x[ii] * 1.0) * 1.0;
  x[ii + 1] -= floor(x[ii + 1] * 1.0) * 1.0;
}

// ------------------------------------------------------------ host side

static inline int blocks_for(long n, int tb)
{
  return (int) ((n + tb - 1) / tb);
}

int f64_create(spss_ctx *ctx)
{
  F64Path *f = new F64Path();
  ctx->f64 = f;
  const long len = (long) ctx->p.n * ctx->s;
  SPSS_TRY(f->state.reserve(len));
  SPSS_TRY(f->rk.reserve(len));
  for (auto &kb : f->k) SPSS_TRY(kb.reserve(len));
  SPSS_TRY(f->td.reserve(len));
  SPSS_TRY(f->det.reserve(len));
  SPSS_TRY(f->caf.reserve(ctx->p.n));
  SPSS_TRY(f->nat_freq.reserve(ctx->p.n));
  SPSS_TRY(f->cell_of.reserve(ctx->p.n));
  SPSS_TRY(f->posf.reserve(ctx->p.n));
  SPSS_TRY(f->csphi.reserve(ctx->p.n));
  SPSS_TRY(f->vl_count.reserve(ctx->p.n));
  SPSS_TRY(f->vl_off.reserve(ctx->p.n + 1));
  SPSS_TRY(f->max2.reserve(1));
  SPSS_TRY(f->partials.reserve(4 * 1024));
  SPSS_CUDA_TRY(cudaMallocHost((void **) &f->h_max2, sizeof(unsigned long long)));
  SPSS_CUDA_TRY(cudaMemsetAsync(f->state.ptr, 0, sizeof(double) * len, ctx->stream));
  for (auto &kb : f->k) SPSS_CUDA_TRY(cudaMemsetAsync(kb.ptr, 0, sizeof(double) * len, ctx->stream));
  SPSS_CUDA_TRY(cudaMemsetAsync(f->caf.ptr, 0, sizeof(double) * ctx->p.n, ctx->stream));
  SPSS_CUDA_TRY(cudaMemsetAsync(f->nat_freq.ptr, 0, sizeof(double) * ctx->p.n, ctx->stream));
  return SPSS_OK;
}

void f64_destroy(spss_ctx *ctx)
{
  F64Path *f = ctx->f64;
  if (!f) return;
  f->state.release();
  f->rk.release();
  for (auto &kb : f->k) kb.release();
  f->td.release();
  f->det.release();
  f->caf.release();
  f->nat_freq.release();
  f->partials.release();
  f->scratch_state.release();
  f->scratch_kprev.release();
  f->scratch_knext.release();
  f->cell_of.release();
  f->posf.release();
  f->csphi.release();
  f->rk2.release();
  f->posf2.release();
  f->csphi2.release();
  if (f->rk4_exec) cudaGraphExecDestroy(f->rk4_exec);
  if (f->rk4_graph) cudaGraphDestroy(f->rk4_graph);
  f->binner.release();
  f->vl_count.release();
  f->vl_off.release();
  f->vl_ent.release();
  f->max2.release();
  if (f->h_max2) cudaFreeHost(f->h_max2);
  delete f;
  ctx->f64 = nullptr;
}

int f64_set_state(spss_ctx *ctx, const double *d_aos)
{
  const long len = (long) ctx->p.n * ctx->s;
  SPSS_CUDA_TRY(cudaMemcpyAsync(ctx->f64->state.ptr, d_aos, sizeof(double) * len, cudaMemcpyDefault,
                                ctx->stream));
  return SPSS_OK;
}

int f64_get_state(spss_ctx *ctx, double *d_aos)
{
  const long len = (long) ctx->p.n * ctx->s;
  SPSS_CUDA_TRY(cudaMemcpyAsync(d_aos, ctx->f64->state.ptr, sizeof(double) * len, cudaMemcpyDefault,
                                ctx->stream));
  return SPSS_OK;
}

int f64_state_ptr(spss_ctx *ctx, const double **d_aos)
{
  *d_aos = ctx->f64->state.ptr;
  return SPSS_OK;
}

static int build_cells(spss_ctx *ctx, const K64 &k, int nc)
{
  F64Path *f = ctx->f64;
  const int tb = 256;
  f64_cell_kernel<<<blocks_for(k.n, tb), tb, 0, ctx->stream>>>(k, f->rk.ptr, nc, f->cell_of.ptr);
  ++ctx->launches;
  SPSS_TRY(check_launch("f64_cell_kernel"));
  SPSS_TRY(f->binner.run(f->cell_of.ptr, k.n, nc * nc, ctx->stream, ctx->launches));
  f->cells_nc = nc;
  return SPSS_OK;
}

static int build_verlet(spss_ctx *ctx, const K64 &k, bool from_cells)
{
  F64Path *f = ctx->f64;
  const int tb = 128;
  if (from_cells)
  {
    SPSS_TRY(build_cells(ctx, k, ctx->nc_verlet));
    f64_verlet_cells_kernel<false><<<blocks_for(k.n, tb), tb, 0, ctx->stream>>>(
        k, f->rk.ptr, ctx->nc_verlet, f->binner.offsets.ptr, f->binner.members.ptr, f->vl_count.ptr, nullptr,
        nullptr);
  } else
  {
    f64_verlet_all_kernel<false><<<blocks_for(k.n, tb), tb, 0, ctx->stream>>>(k, f->rk.ptr, f->vl_count.ptr,
                                                                               nullptr, nullptr);
  }
  ++ctx->launches;
  SPSS_TRY(check_launch("f64_verlet_count"));
  SPSS_TRY(f->binner.scanner.run(f->vl_count.ptr, f->vl_off.ptr, k.n, ctx->stream, ctx->launches));
  int total = 0;
  SPSS_CUDA_TRY(cudaMemcpyAsync(&total, f->vl_off.ptr + k.n, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  SPSS_TRY(f->vl_ent.reserve(total > 0 ? total : 1));
  if (from_cells)
  {
    f64_verlet_cells_kernel<true><<<blocks_for(k.n, tb), tb, 0, ctx->stream>>>(
        k, f->rk.ptr, ctx->nc_verlet, f->binner.offsets.ptr, f->binner.members.ptr, nullptr, f->vl_off.ptr,
        f->vl_ent.ptr);
  } else
  {
    f64_verlet_all_kernel<true><<<blocks_for(k.n, tb), tb, 0, ctx->stream>>>(k, f->rk.ptr, nullptr, f->vl_off.ptr,
                                                                              f->vl_ent.ptr);
  }
  ++ctx->launches;
  SPSS_TRY(check_launch("f64_verlet_fill"));
  f->vl_total = total;
  f->vl_built = 1;
  return SPSS_OK;
}

int f64_evaluate(spss_ctx *ctx, int variant, const double *d_state, const double *d_kprev, double *d_knext,
                 double k_coef, double dt)
{
  F64Path *f = ctx->f64;
  variant = variant_for(ctx, variant);
  if (variant < SPSS_VARIANT_ALL_PAIRS || variant > SPSS_VARIANT_GLOBAL_FIELD) return SPSS_ERR_INVALID_ARGUMENT;
  if (variant == SPSS_VARIANT_GLOBAL_FIELD && ctx->p.model != 1) return SPSS_ERR_NOT_SUPPORTED;
  const K64 k = make_k64(ctx);
  const long len = (long) k.n * k.s;
  const int tb = 256;
  if (variant == SPSS_VARIANT_ALL_PAIRS)
    f64_stage_posf_kernel<<<blocks_for(k.n, tb), tb, 0, ctx->stream>>>(k, d_state, d_kprev, f->rk.ptr, f->posf.ptr,
                                                                       f->csphi.ptr, k_coef, dt);
  else
    f64_stage_kernel<<<blocks_for(len, tb), tb, 0, ctx->stream>>>(d_state, d_kprev, f->rk.ptr, len, k_coef, dt);
  ++ctx->launches;
  SPSS_TRY(check_launch("f64_stage_kernel"));
  if (k.higher_order) SPSS_CUDA_TRY(cudaMemsetAsync(f->caf.ptr, 0, sizeof(double) * k.n, ctx->stream));
  switch (variant)
  {
    case SPSS_VARIANT_ALL_PAIRS:
      f64_allpairs_kernel<<<blocks_for(32L * k.n, 128), 128, 0, ctx->stream>>>(
          k, f->rk.ptr, f->posf.ptr, f->csphi.ptr, d_knext, f->caf.ptr, NextStage{});
      ++ctx->launches;
      return check_launch("f64_allpairs_kernel");
    case SPSS_VARIANT_LINKED_LIST:
      SPSS_TRY(build_cells(ctx, k, ctx->nc));
      f64_linked_list_kernel<<<blocks_for(k.n, 128), 128, 0, ctx->stream>>>(
          k, f->rk.ptr, ctx->nc, f->binner.offsets.ptr, f->binner.members.ptr, d_knext, f->caf.ptr);
      ++ctx->launches;
      return check_launch("f64_linked_list_kernel");
    case SPSS_VARIANT_VERLET:
    case SPSS_VARIANT_LINKED_LIST_VERLET:
      if (ctx->should_update_lists)
      {
        SPSS_TRY(build_verlet(ctx, k, variant == SPSS_VARIANT_LINKED_LIST_VERLET));
        ctx->should_update_lists = 0;
        ++ctx->list_builds;
      }
      ctx->uses_verlet_list = 1;
      f64_verlet_pairs_kernel<<<blocks_for(k.n, 128), 128, 0, ctx->stream>>>(k, f->rk.ptr, f->vl_off.ptr,
                                                                             f->vl_ent.ptr, d_knext, f->caf.ptr);
      ++ctx->launches;
      return check_launch("f64_verlet_pairs_kernel");
    case SPSS_VARIANT_GLOBAL_FIELD:
    {
      const int nparts = std::min(1024, blocks_for(k.n, 256));
      f64_field_partials_kernel<<<nparts, 256, 0, ctx->stream>>>(k, f->rk.ptr, f->partials.ptr);
      ++ctx->launches;
      SPSS_TRY(check_launch("f64_field_partials_kernel"));
      f64_field_apply_kernel<<<blocks_for(k.n, 256), 256, 0, ctx->stream>>>(k, f->rk.ptr, f->partials.ptr, nparts,
                                                                            f->nat_freq.ptr, d_knext, f->caf.ptr);
      ++ctx->launches;
      return check_launch("f64_field_apply_kernel");
    }
  }
  return SPSS_ERR_INVALID_ARGUMENT;
}

int f64_max_displacement(spss_ctx *ctx, const double *d_td, double *max2_out)
{
  F64Path *f = ctx->f64;
  SPSS_CUDA_TRY(cudaMemsetAsync(f->max2.ptr, 0, sizeof(unsigned long long), ctx->stream));
  const int nb = std::min(1024, blocks_for(ctx->p.n, 256));
  f64_max2_kernel<<<nb, 256, 0, ctx->stream>>>(d_td, ctx->p.n, ctx->s, f->max2.ptr);
  ++ctx->launches;
  SPSS_TRY(check_launch("f64_max2_kernel"));
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->h_max2, f->max2.ptr, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  unsigned long long bits = *f->h_max2;
  std::memcpy(max2_out, &bits, sizeof(double));
  return SPSS_OK;
}

static NoiseKey noise_key(const spss_ctx *ctx, unsigned long long step)
{
  NoiseKey nk;
  nk.seed = ctx->p.seed;
  nk.replica = ctx->p.replica;
  nk.step = step;
  return nk;
}

int f64_step(spss_ctx *ctx, int stepper, double t, double dt)
{
  (void) t;
  F64Path *f = ctx->f64;
  const int n = ctx->p.n, s = ctx->s;
  const long len = (long) n * s;
  const int variant = ctx->p.variant;
  const int tb = 256;
  if (stepper == SPSS_STEPPER_RK4 && variant_for(ctx, variant) == SPSS_VARIANT_ALL_PAIRS && !ctx->higher_order)
  {
    // four all-pairs evaluations, each pair kernel also writing the next
    // stage (x + 0.5 dt k1, x + 0.5 dt k2, x + dt k3) into the other stage
    // buffers: six kernels instead of nine, the same arithmetic
    double *x = f->state.ptr;
    const K64 k = make_k64(ctx);
    SPSS_TRY(f->rk2.reserve(len));
    SPSS_TRY(f->posf2.reserve(n));
    SPSS_TRY(f->csphi2.reserve(n));
    f64_stage_posf_kernel<<<blocks_for(n, tb), tb, 0, ctx->stream>>>(k, x, f->k[0].ptr, f->rk.ptr, f->posf.ptr,
                                                                     f->csphi.ptr, 0.0, dt);
    ++ctx->launches;
    SPSS_TRY(check_launch("f64_stage_posf_kernel"));
    double *rk[2] = {f->rk.ptr, f->rk2.ptr};
    float2 *pf[2] = {f->posf.ptr, f->posf2.ptr};
    double2 *cs[2] = {f->csphi.ptr, f->csphi2.ptr};
    const double coef[3] = {0.5, 0.5, 1.0};
    for (int e = 0; e < 4; ++e)
    {
      const int a = e & 1, b = a ^ 1;
      const NextStage next = e < 3 ? NextStage{x, coef[e], dt, rk[b], pf[b], cs[b]} : NextStage{};
      f64_allpairs_kernel<<<blocks_for(32L * n, 128), 128, 0, ctx->stream>>>(k, rk[a], pf[a], cs[a], f->k[e].ptr,
                                                                            f->caf.ptr, next);
      ++ctx->launches;
      SPSS_TRY(check_launch("f64_allpairs_kernel"));
    }
    f64_rk4_combine_kernel<<<blocks_for(len, tb), tb, 0, ctx->stream>>>(x, f->k[0].ptr, f->k[1].ptr, f->k[2].ptr,
                                                                        f->k[3].ptr, f->td.ptr, len, dt);
    ++ctx->launches;
    SPSS_TRY(check_launch("f64_rk4_combine_kernel"));
  } else if (stepper == SPSS_STEPPER_RK4)
  {
    double *x = f->state.ptr;
    SPSS_TRY(f64_evaluate(ctx, variant, x, f->k[0].ptr, f->k[0].ptr, 0.0, dt));
    SPSS_TRY(f64_evaluate(ctx, variant, x, f->k[0].ptr, f->k[1].ptr, 0.5, dt));
    SPSS_TRY(f64_evaluate(ctx, variant, x, f->k[1].ptr, f->k[2].ptr, 0.5, dt));
    SPSS_TRY(f64_evaluate(ctx, variant, x, f->k[2].ptr, f->k[3].ptr, 1.0, dt));
    f64_rk4_combine_kernel<<<blocks_for(len, tb), tb, 0, ctx->stream>>>(x, f->k[0].ptr, f->k[1].ptr, f->k[2].ptr,
                                                                        f->k[3].ptr, f->td.ptr, len, dt);
    ++ctx->launches;
    SPSS_TRY(check_launch("f64_rk4_combine_kernel"));
  } else
  {
    const NoiseKey nk = noise_key(ctx, ctx->step_counter);
    SPSS_CUDA_TRY(cudaMemsetAsync(f->det.ptr, 0, sizeof(double) * len, ctx->stream));
    if (stepper == SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA) ctx->higher_order = 1;
    SPSS_TRY(f64_evaluate(ctx, variant, f->state.ptr, f->det.ptr, f->det.ptr, 0.0, dt));
    const double sqrt_dt = std::sqrt(dt);
    if (stepper == SPSS_STEPPER_STOCHASTIC_EULER)
    {
      if (ctx->p.model == 2)
        f64_se2_kernel<<<blocks_for(n, tb), tb, 0, ctx->stream>>>(f->state.ptr, f->det.ptr, f->td.ptr, n, dt,
                                                                  sqrt_dt, std::sqrt(2.0 * ctx->p.D_r),
                                                                  std::sqrt(2.0 * ctx->p.D_phi), nk);
      else
        f64_se1_kernel<<<blocks_for(n, tb), tb, 0, ctx->stream>>>(f->state.ptr, f->det.ptr, f->td.ptr, n, dt,
                                                                  sqrt_dt, std::sqrt(2.0 * ctx->p.D_phi), nk);
    } else if (stepper == SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA)
    {
      const double dt15 = std::pow(dt, 1.5), inv_sqrt3 = 1.0 / std::sqrt(3.0);
      if (ctx->p.model == 1)
        f64_srk1_kernel<<<blocks_for(n, tb), tb, 0, ctx->stream>>>(f->state.ptr, f->det.ptr, f->caf.ptr, f->td.ptr,
                                                                   n, dt, sqrt_dt, dt15, inv_sqrt3,
                                                                   std::sqrt(2.0 * ctx->p.D_phi), ctx->p.xi, nk);
      else
        f64_srk2_kernel<<<blocks_for(n, tb), tb, 0, ctx->stream>>>(
            f->state.ptr, f->det.ptr, f->caf.ptr, f->td.ptr, n, dt, sqrt_dt, dt15, inv_sqrt3,
            std::sqrt(2.0 * ctx->p.D_r), std::sqrt(2.0 * ctx->p.D_phi), ctx->p.xi_r, ctx->p.xi_phi, ctx->p.v0, nk);
    } else
    {
      return SPSS_ERR_INVALID_ARGUMENT;
    }
    ++ctx->launches;
    SPSS_TRY(check_launch("f64 stepper kernel"));
    ++ctx->step_counter;
  }
  if (ctx->uses_verlet_list)
  {
    double max2 = 0.0;
    SPSS_TRY(f64_max_displacement(ctx, f->td.ptr, &max2));
    SPSS_TRY(host_calculate_max_displacement(ctx, max2));
  }
  return SPSS_OK;
}

// nsteps RK4 steps: one step runs as it is (sizing every buffer), the rest
// replay that step captured as a CUDA graph — RK4 draws no noise and, without
// a Verlet list, needs no host decision between steps.  The state is
// identical to nsteps single steps.  Other steppers and Verlet contexts step
// one by one.
int f64_steps(spss_ctx *ctx, int stepper, double t0, double dt, int nsteps)
{
  F64Path *f = ctx->f64;
  double t = t0;
  const bool graphable = stepper == SPSS_STEPPER_RK4 && !ctx->uses_verlet_list &&
                         variant_for(ctx, ctx->p.variant) != SPSS_VARIANT_VERLET &&
                         variant_for(ctx, ctx->p.variant) != SPSS_VARIANT_LINKED_LIST_VERLET;
  if (!graphable || nsteps < 3)
  {
    for (int k = 0; k < nsteps; ++k)
    {
      t += dt;
      SPSS_TRY(f64_step(ctx, stepper, t, dt));
    }
    return SPSS_OK;
  }
  t += dt;
  SPSS_TRY(f64_step(ctx, stepper, t, dt));
  if (!f->rk4_exec || f->rk4_dt != dt || f->rk4_higher_order != ctx->higher_order)
  {
    if (f->rk4_exec) cudaGraphExecDestroy(f->rk4_exec);
    if (f->rk4_graph) cudaGraphDestroy(f->rk4_graph);
    f->rk4_exec = nullptr;
    f->rk4_graph = nullptr;
    cudaStream_t work = ctx->stream;
    ctx->stream = ctx->own_stream;  // capture needs a non-legacy stream
    const unsigned long long launches0 = ctx->launches;
    SPSS_CUDA_TRY(cudaStreamSynchronize(work));
    int rc = SPSS_OK;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = SPSS_ERR_CUDA;
    if (rc == SPSS_OK) rc = f64_step(ctx, stepper, t + dt, dt);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->stream = work;
    f->rk4_launches = ctx->launches - launches0;
    ctx->launches = launches0;
    if (rc == SPSS_OK && e != cudaSuccess) rc = SPSS_ERR_CUDA;
    if (rc == SPSS_OK && cudaGraphInstantiate(&f->rk4_exec, g, 0) != cudaSuccess) rc = SPSS_ERR_CUDA;
    if (rc != SPSS_OK)
    {
      cudaGetLastError();
      if (g) cudaGraphDestroy(g);
      f->rk4_exec = nullptr;
      return rc;
    }
    f->rk4_graph = g;
    f->rk4_dt = dt;
    f->rk4_higher_order = ctx->higher_order;
  }
  for (int k = 1; k < nsteps; ++k) SPSS_CUDA_TRY(cudaGraphLaunch(f->rk4_exec, ctx->stream));
  ctx->launches += f->rk4_launches * (unsigned long long) (nsteps - 1);
  return SPSS_OK;
}

int f64_noise(spss_ctx *ctx, int stepper, unsigned long long step, double *d_out)
{
  const int per = normals_per_particle(ctx->p.model, stepper);
  if (per == 0) return SPSS_OK;
  f64_noise_kernel<<<blocks_for(ctx->p.n, 256), 256, 0, ctx->stream>>>(d_out, ctx->p.n, per, noise_key(ctx, step));
  ++ctx->launches;
  return check_launch("f64_noise_kernel");
}

int f64_complementary_force(spss_ctx *ctx, double *d_out)
{
  SPSS_CUDA_TRY(cudaMemcpyAsync(d_out, ctx->f64->caf.ptr, sizeof(double) * ctx->p.n, cudaMemcpyDeviceToDevice,
                                ctx->stream));
  return SPSS_OK;
}

int f64_set_natural_frequencies(spss_ctx *ctx, const double *d_freqs)
{
  SPSS_CUDA_TRY(cudaMemcpyAsync(ctx->f64->nat_freq.ptr, d_freqs, sizeof(double) * ctx->p.n,
                                cudaMemcpyDeviceToDevice, ctx->stream));
  return SPSS_OK;
}

int f64_lists(spss_ctx *ctx, int **pll, int **cell_off, int **cell_mem, int *ncell, int **vl_off, int **vl_ent,
              long *vl_total)
{
  F64Path *f = ctx->f64;
  *pll = f->cells_nc ? f->cell_of.ptr : nullptr;
  *cell_off = f->cells_nc ? f->binner.offsets.ptr : nullptr;
  *cell_mem = f->cells_nc ? f->binner.members.ptr : nullptr;
  *ncell = f->cells_nc * f->cells_nc;
  *vl_off = f->vl_built ? f->vl_off.ptr : nullptr;
  *vl_ent = f->vl_built ? f->vl_ent.ptr : nullptr;
  *vl_total = f->vl_built ? f->vl_total : 0;
  return SPSS_OK;
}

int f64_apply_pbc(spss_ctx *ctx)
{
  f64_pbc_kernel<<<blocks_for(ctx->p.n, 256), 256, 0, ctx->stream>>>(ctx->f64->state.ptr, ctx->p.n, ctx->s);
  ++ctx->launches;
  return check_launch("f64_pbc_kernel");
}

}  // namespace spss
