// GB300 fast path: fixed-point positions, FP32 pair and stage arithmetic,
// fused pair sums + stochastic stepper update + Philox noise.
//
// Representation (slot order; slots are re-sorted by cell at every rebuild):
//   rec[2][n]  uint4 {x_hi, y_hi, cos phi, sin phi}: the record a neighbour
//              gathers; double-buffered, a step reads rec[parity] (neighbours
//              see the previous state) and writes rec[parity ^ 1]
//   aux[2][n]  uint4 {x_lo, y_lo, phase, omega}, double-buffered with rec
//   vel[n]     float2 {v_x, v_y} (second-order model), updated in place
//   pid[n]     original particle index (noise counter, output order); inv[n]
//              its inverse
//   img[n], turns[n]  box crossings and 2*pi turns of the phase, indexed by
//              original index (they change rarely, so the slot re-sort of a
//              rebuild does not move them)
// x = img + (x_hi * 2^32 + x_lo) * 2^-64 (unit box), phase = 2*pi*(turns + phase * 2^-32).
//
// The owner of a particle evaluates cos and sin of its phase once per step and
// stores them in its record, so a pair costs no transcendental:
// sum_j sin(phi_j - phi_i) = cos phi_i sum_j sin phi_j - sin phi_i sum_j cos phi_j.
//
// FP64 appears only where the result must not depend on FP32 rounding: the
// exact cutoff decision inside a guard band around r = rho (a few pairs per
// step), the accumulated Verlet displacement and the upload/download
// conversions.  GB300 runs FP64 at about 1/70 of its FP32 rate.
//
// Reference semantics mirrored: ParticleSystemFirstOrder.cpp / ParticleSystemFirstOrderPtr.cpp
// (pair sums, isolated particles keep zero torque derivative in SE/SRK),
// ParticleSystemSecondOrder.cpp, StochasticEulerStepper.hpp:33-51,
// StochasticEulerStepperPtr.hpp:40-73, StochasticRungeKuttaStepperPtr.hpp:40-76,
// CalculateMaxDisplacement ParticleSystemFirstOrder.cpp:670-696.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <utility>

#include "spss_internal.cuh"

namespace spss
{

constexpr int kTB = 256;

struct FastControl
{
  unsigned long long step;  // Philox step counter of the next stochastic step
  double acc;               // accumulated displacement of system 0 (FP64)
  int parity;               // current rec/aux buffer
  int rebuild;              // lists (and slot order) rebuilt before the next evaluation
  int cells_fresh;          // cell ids of the current slots were written by the last cell-list step
  int overflow;             // largest Verlet count seen beyond capacity (0: none)
  int rebuilds;             // number of rebuilds performed
  int error;                // bit 0: displacement too large for the fixed-point increment; bit 1: staging
                            // timeout; bit 2: stencil cell outside the staged segments; bit 3: the
                            // device launch of the rebuild graph was refused
  int uses_verlet;
  int tile_next;            // work counter of the persistent tile kernel
  int triggered;            // the last step's displacement trigger fired (its rebuild may already be done)
  long long sample_every;   // order-parameter samples after steps that are multiples of this (0: none)
  long long sample_from;    // ... and not before this step
};

// Per-system Verlet trigger state (CalculateMaxDisplacement of each system).
struct SysControl
{
  double acc;              // accumulated displacement (FP64)
  unsigned int max2_bits;  // max |dr|^2 of the step, FP32 bits (non-negative floats order as ints)
  int rebuild;             // this system's lists are rebuilt before the next step (per-system rebuilds)
};

// FastControl::rebuild: no rebuild, every system, or the systems whose own
// trigger fired (SysControl::rebuild; batches of Verlet-list systems).
enum
{
  REBUILD_NONE = 0,
  REBUILD_ALL = 1,
  REBUILD_FLAGGED = 2
};

// One independent system of a context (a context holds one or a batch of
// them; each is the reference's particle system on its own unit box).  Its
// particles are the slots [first, first + n) in every slot order, its cells
// the global cells [cell0, cell0 + nc^2), its tiles [tile0, tile0 + ntiles).
struct SysParams
{
  int n, first, nc, cell0;
  int tile0, ntiles, index, replica;
  float v0, xi, xi_r, xi_phi, sigma, ca, sa, rho2_f;
  float band_f, rmax2_f, b_r, b_phi;
  double rho2_d, half_skin;
};

enum Kind
{
  KIND_ALL_PAIRS = 0,
  KIND_GLOBAL = 3,  // global polar order field (first order): no lists, slot = original index
  KIND_CELLS = 1,
  KIND_VERLET = 2
};

// Launch parameters: context-wide fields, plus the fields of one system
// (nc .. replica), which kernels that work on several systems overwrite from
// the system table (with_system).
struct FastParams
{
  int n, nc, cap, model;      // n: slots of the whole context
  int kind, always_rebuild, tile_cells, persistent;
  int nsys, ntiles, first, sub_n;
  int cell0, sys, selective, pad1;  // selective: per-system rebuilds (batches of Verlet-list systems)
  float v0, xi, xi_r, xi_phi, sigma, ca, sa;
  float rho2_f, band_f, rmax2_f;
  double rho2_d, half_skin;
  float dt, sqdt, half_dt2, half_dt15, inv_sqrt3, b_r, b_phi;
  uint64_t seed;
  uint32_t replica;
  uint32_t kx[10], ky[10];  // Philox round keys of `seed`, the same for every particle
};

struct FastBuffers
{
  uint4 *rec0, *rec1;
  uint4 *aux0, *aux1;
  float2 *vel, *vel_tmp;
  unsigned *pid, *pid_tmp, *inv;
  int2 *img;   // box crossings, by original index
  int *turns;  // 2 pi turns of the phase, by original index
  int *cell_of, *cell_sorted;
  const int *cell_off;
  const int *order;
  short *vl;
  int *vl_cnt;
  float *nu;             // natural frequencies (global field), slot = original index
  double *field;         // Z = <e^{i phi}>, W = <omega e^{i phi}> and derived values (global field)
  double *field_partial; // block partials of the field sums
  const SysParams *sys;  // system table
  const int *sys_of;     // system of each slot (equivalently of each original index)
  const int *tile_sys;   // system of each tile
  SysControl *sysctl;
  int *tile_maxcnt;  // longest list of each tile (rows to stage)
  void *tiles;       // TileLayout of every tile, written at rebuild
  FastControl *ctrl;
};

// How a step graph does the list rebuild: under a conditional node at the
// start of the step (GRAPH_CONDITIONAL), tail-launched as a device graph by the
// control kernel when the trigger fires (GRAPH_DEVICE), unconditionally at the
// start of every step (GRAPH_ALWAYS: cell lists), or not at all (GRAPH_NONE:
// kinds without lists or trigger).  Rebuilds requested from the host run
// before the first graph step in the last three forms.
enum
{
  GRAPH_CONDITIONAL = 0,
  GRAPH_DEVICE = 1,
  GRAPH_ALWAYS = 2,
  GRAPH_NONE = 3
};

// Device copy of the stepping state, for restoring it after trial steps.
struct Snapshot
{
  DeviceArray<uint4> rec[2], aux[2];
  DeviceArray<float2> vel;
  DeviceArray<unsigned> pid, inv;
  DeviceArray<int2> img;
  DeviceArray<int> turns;
  DeviceArray<SysControl> sysctl;
  DeviceArray<FastControl> ctrl;
  void release()
  {
    for (int b = 0; b < 2; ++b)
    {
      rec[b].release();
      aux[b].release();
    }
    vel.release();
    pid.release();
    inv.release();
    img.release();
    turns.release();
    sysctl.release();
    ctrl.release();
  }
};

// FP64 sums of one chunk of a system: cos phi, sin phi, v_x/|v|, v_y/|v|.
struct __align__(16) OrderSums
{
  double c, s, vx, vy;
};

struct GraphEntry
{
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  // the rebuild as a device-launchable graph, tail-launched by the step's
  // control kernel when the trigger fires (null: the step graph holds the
  // rebuild under a conditional node instead)
  cudaGraphExec_t rebuild_exec = nullptr;
  cudaGraph_t rebuild_graph = nullptr;
  int per_step = 0;     // kernels of the unconditional part
  int per_rebuild = 0;  // kernels of the rebuild
  int form = 0;         // GRAPH_* below
  void release()
  {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (rebuild_exec) cudaGraphExecDestroy(rebuild_exec);
    if (rebuild_graph) cudaGraphDestroy(rebuild_graph);
    *this = GraphEntry();
  }
};

struct FastPath
{
  DeviceArray<uint4> rec[2], aux[2];
  DeviceArray<float2> vel, vel_tmp;
  DeviceArray<unsigned> pid, pid_tmp, inv;
  DeviceArray<int2> img;
  DeviceArray<int> turns, cell_of, cell_sorted, vl_cnt, tile_maxcnt;
  DeviceArray<short> vl;
  DeviceArray<unsigned char> tiles;
  DeviceArray<SysParams> sys;
  DeviceArray<int> sys_of, tile_sys;
  DeviceArray<SysControl> sysctl;
  DeviceArray<float> nu;
  DeviceArray<double> field, field_partial;
  std::vector<SysParams> h_sys;
  int nsys = 1;
  int total_cells = 1;
  int ntiles = 0;
  int tile_cells = 32;
  int persistent = 0;
  int persistent_grid = 0;
  Binner binner;
  FastControl *ctrl = nullptr;    // device
  FastControl *h_ctrl = nullptr;  // pinned mirror
  int kind = KIND_CELLS;
  // Verlet bookkeeping without lists: a Verlet-list context whose radius
  // leaves fewer than three cells per side evaluates all pairs every step and
  // keeps the displacement trigger (uses_verlet_list, accumulated displacement).
  bool trigger_only = false;
  int nc_build = 1;
  int cap = 0;
  bool have_state = false;
  bool perm_valid = false;
  std::map<std::tuple<int, double, int>, GraphEntry> graphs;  // (stepper, dt, with sampling)
  bool device_rebuild = true;  // rebuilds tail-launched as device graphs (cleared if this device refuses)
  // set while a cell-list step graph is captured: its kernels after the first
  // are launched as a programmatic-dependent chain (each begins with pdl_enter)
  bool chain = false;
  // per-system order parameters and their time averages
  DeviceArray<OrderSums> order_partial;
  DeviceArray<int2> order_items;   // (system, first slot) of every chunk, systems in order
  DeviceArray<int> order_first;    // first chunk of every system, nsys + 1 entries
  DeviceArray<double> order_out, stats;
  int order_chunks = 1;  // chunks of all systems
  int order_grid = 1;
  Snapshot snap;
};

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ uint64_t join64(uint32_t hi, uint32_t lo)
{
  return ((uint64_t) hi << 32) | lo;
}

// The launch parameters with the fields of system S.
__device__ __forceinline__ FastParams with_system(const FastParams &P, const SysParams &S)
{
  FastParams Q = P;
  Q.nc = S.nc;
  Q.first = S.first;
  Q.sub_n = S.n;
  Q.cell0 = S.cell0;
  Q.sys = S.index;
  Q.v0 = S.v0;
  Q.xi = S.xi;
  Q.xi_r = S.xi_r;
  Q.xi_phi = S.xi_phi;
  Q.sigma = S.sigma;
  Q.ca = S.ca;
  Q.sa = S.sa;
  Q.rho2_f = S.rho2_f;
  Q.band_f = S.band_f;
  Q.rmax2_f = S.rmax2_f;
  Q.b_r = S.b_r;
  Q.b_phi = S.b_phi;
  Q.rho2_d = S.rho2_d;
  Q.half_skin = S.half_skin;
  Q.replica = (uint32_t) S.replica;
  return Q;
}

// round-toward-zero f * 2^64 as a signed integer, exact for the 24-bit
// mantissa; |f| < 0.5 (one step never moves a particle half a box).
__device__ __forceinline__ long long fix64_of(float f, int &err)
{
  if (!(fabsf(f) < 0.5f))
  {
    err = 1;
    return 0;
  }
  return __float2ll_rz(__fmul_rn(f, 18446744073709551616.0f));  // exact scaling by 2^64, then truncation
}

// X += dX on the periodic unit box; `carry` receives the box crossing (-1, 0, 1).
__device__ __forceinline__ uint64_t advance(uint64_t X, long long dX, int &carry)
{
  const uint64_t Y = X + (uint64_t) dX;
  carry = (dX > 0 && Y < X) ? 1 : ((dX < 0 && Y > X) ? -1 : 0);
  return Y;
}

__device__ __forceinline__ uint32_t advance_phase(uint32_t P, float dphi, int &carry, int &err)
{
  // 2^32 / (2 pi)
  const float q = dphi * 683565275.5764316f;
  carry = 0;
  if (!(fabsf(q) < 2.1e9f))
  {
    err = 1;
    return P;
  }
  const int d = __float2int_rn(q);
  const uint32_t R = P + (uint32_t) d;
  carry = (d > 0 && R < P) ? 1 : ((d < 0 && R > P) ? -1 : 0);
  return R;
}

// sin and cos of the fixed-point phase P (one turn = 2^32).  The nearest
// quarter turn comes exactly from the top bits; the remainder is the angle
// theta = 2 pi r 2^-32 in [-pi/4, pi/4), where sin and cos are an odd degree-7
// and an even degree-8 polynomial in theta (coefficients fitted by weighted
// least squares on Chebyshev nodes of theta^2, rounded to float).  The
// result is within 1e-7 of the exact sin and cos of the phase over all 2^32
// phases (the rounding of theta to float is the larger part); the quarter-turn
// rotation is exact.  Rounding is spelled out so every copy gives the same bits.
__device__ __forceinline__ void phase_sincos(uint32_t P, float &s, float &c)
{
  const uint32_t qd = (P + 0x20000000u) >> 30;  // nearest quarter turn (mod 4)
  const int r = (int) (P - (qd << 30));         // [-2^29, 2^29)
  const float th = __fmul_rn((float) r, 1.4629180792671596e-9f);  // 2 pi / 2^32
  const float t2 = __fmul_rn(th, th);
  const float ps = fmaf(th, __fmul_rn(t2, fmaf(t2, fmaf(t2, -1.9520212663337588e-4f, 8.332204073667526e-3f),
                                               -0.16666655242443085f)),
                        th);
  const float pc = fmaf(t2, fmaf(t2, fmaf(t2, fmaf(t2, 2.4394103093072772e-5f, -1.3886808883398771e-3f),
                                          4.166662320494652e-2f),
                                 -0.5f),
                        1.0f);
  // rotate by qd quarter turns: (sin, cos) = (ps, pc), (pc, -ps), (-ps, -pc), (-pc, ps)
  const float a = (qd & 1u) ? pc : ps;
  const float b = (qd & 1u) ? ps : pc;
  s = (qd & 2u) ? -a : a;
  c = ((qd + 1u) & 2u) ? -b : b;
}

__device__ __forceinline__ int cell_of_fix(uint64_t X, uint64_t Y, int nc)
{
  const int cx = (int) __umul64hi(X, (uint64_t) nc);
  const int cy = (int) __umul64hi(Y, (uint64_t) nc);
  return cy * nc + cx;
}

__device__ __forceinline__ int wrap_cell(int c, int nc)
{
  return c < 0 ? nc - 1 : (c >= nc ? 0 : c);
}

struct Acc
{
  float ss, sc, ws, wc;
  int card;
};

// One candidate pair: FP32 distance from the 32-bit high words (exact minimum
// image by integer subtraction); inside the guard band the decision is
// recomputed in FP64 from the full 64-bit positions, so it equals the FP64
// decision for these positions.
// The FP64 cutoff decision from the full 64-bit positions, for a pair inside
// the guard band (a few pairs per step).
__device__ __forceinline__ bool exact_within_inline(uint32_t xh, uint32_t yh, uint32_t xl, uint32_t yl, uint64_t Xi,
                                                   uint64_t Yi, double rho2)
{
  const double ex = (double) (long long) (join64(xh, xl) - Xi) * 5.421010862427522e-20;
  const double ey = (double) (long long) (join64(yh, yl) - Yi) * 5.421010862427522e-20;
  return __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)) <= rho2;
}

// Out of line, for the stencil scans: keeps their loops small in the
// instruction cache (the Verlet-list walk keeps the inline form, which costs
// no call).
__device__ __noinline__ bool exact_within(uint32_t xh, uint32_t yh, uint32_t xl, uint32_t yl, uint64_t Xi,
                                          uint64_t Yi, double rho2)
{
  return exact_within_inline(xh, yh, xl, yl, Xi, Yi, rho2);
}

template<bool OUTLINE>
__device__ __forceinline__ bool in_range(const FastParams &P, const uint4 &ri, uint64_t Xi, uint64_t Yi,
                                         const uint4 &rj, const uint4 *__restrict__ aux, int j)
{
  const float dx = (float) (int) (rj.x - ri.x);
  const float dy = (float) (int) (rj.y - ri.y);
  const float d2 = fmaf(dx, dx, dy * dy);
  bool in = d2 <= P.rho2_f;
  if (fabsf(d2 - P.rho2_f) <= P.band_f)
  {
    const uint2 l = __ldg(reinterpret_cast<const uint2 *>(&aux[j]));
    in = OUTLINE ? exact_within(rj.x, rj.y, l.x, l.y, Xi, Yi, P.rho2_d)
                 : exact_within_inline(rj.x, rj.y, l.x, l.y, Xi, Yi, P.rho2_d);
  }
  return in;
}

__device__ __forceinline__ void accumulate(Acc &a, const uint4 &rj, float wj)
{
  const float cj = __uint_as_float(rj.z), sj = __uint_as_float(rj.w);
  a.sc += cj;
  a.ss += sj;
  a.wc = fmaf(wj, cj, a.wc);
  a.ws = fmaf(wj, sj, a.ws);
  a.card += 1;
}

template<bool OMEGA, bool OUTLINE>
__device__ __forceinline__ void candidate(const FastParams &P, const uint4 &ri, uint64_t Xi, uint64_t Yi,
                                          const uint4 *__restrict__ rec, const uint4 *__restrict__ aux, int j, Acc &a)
{
  const uint4 rj = __ldg(&rec[j]);
  if (in_range<OUTLINE>(P, ri, Xi, Yi, rj, aux, j)) accumulate(a, rj, OMEGA ? __uint_as_float(__ldg(&aux[j].w)) : 0.0f);
}

// Four list entries at a time: the entry loads, then the record loads, then
// the omega loads of the pairs in range are issued together, so a thread has
// several gathers in flight instead of a chain of dependent ones.
template<bool OMEGA, bool OUTLINE>
__device__ __forceinline__ void candidates4(const FastParams &P, const uint4 &ri, uint64_t Xi, uint64_t Yi,
                                            const uint4 *__restrict__ rec, const uint4 *__restrict__ aux,
                                            const int j[4], Acc &a)
{
  uint4 r[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) r[u] = __ldg(&rec[j[u]]);
  bool in[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) in[u] = in_range<OUTLINE>(P, ri, Xi, Yi, r[u], aux, j[u]);
  float w[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) w[u] = (OMEGA && in[u]) ? __uint_as_float(__ldg(&aux[j[u]].w)) : 0.0f;
#pragma unroll
  for (int u = 0; u < 4; ++u)
    if (in[u]) accumulate(a, r[u], w[u]);
}

// ---------------------------------------------------------------- conversions

// A block's contiguous AoS rows move between global (possibly host) memory
// and shared memory in 16-byte pieces when the array allows it, so that reads
// and writes over the host link are whole coalesced lines.
__device__ __forceinline__ void rows_to_shared(const double *__restrict__ g, double *sh, int count)
{
  if (((uintptr_t) g & 15) == 0)
  {
    const double2 *g2 = reinterpret_cast<const double2 *>(g);
    double2 *s2 = reinterpret_cast<double2 *>(sh);
    for (int i = threadIdx.x; i < count / 2; i += blockDim.x) s2[i] = g2[i];
    if ((count & 1) && threadIdx.x == 0) sh[count - 1] = g[count - 1];
  } else
  {
    for (int i = threadIdx.x; i < count; i += blockDim.x) sh[i] = g[i];
  }
}

__device__ __forceinline__ void rows_from_shared(double *__restrict__ g, const double *sh, int count)
{
  if (((uintptr_t) g & 15) == 0)
  {
    double2 *g2 = reinterpret_cast<double2 *>(g);
    const double2 *s2 = reinterpret_cast<const double2 *>(sh);
    for (int i = threadIdx.x; i < count / 2; i += blockDim.x) g2[i] = s2[i];
    if ((count & 1) && threadIdx.x == 0) g[count - 1] = sh[count - 1];
  } else
  {
    for (int i = threadIdx.x; i < count; i += blockDim.x) g[i] = sh[i];
  }
}

// Upload from reference AoS, one thread per original index p (its block's
// rows read as one coalesced chunk), scattered to the particle's slot inv[p]
// (identity when no slot order exists yet).
__global__ void fast_upload_kernel(const double *__restrict__ x, int n, int s, int model, int perm_valid,
                                   FastBuffers B)
{
  extern __shared__ double rows[];
  const int p0 = blockIdx.x * blockDim.x;
  const int count = min((int) blockDim.x, n - p0) * s;
  rows_to_shared(x + (long) s * p0, rows, count);
  __syncthreads();
  const int p = p0 + threadIdx.x;
  if (p >= n) return;
  const int par = B.ctrl->parity;
  unsigned q = (unsigned) p;
  if (perm_valid)
  {
    q = B.inv[p];
  } else
  {
    B.pid[p] = (unsigned) p;
    B.inv[p] = (unsigned) p;
  }
  const double *st = rows + s * threadIdx.x;
  int2 im;
  uint64_t X, Y;
  {
    const double fx = floor(st[0]), fy = floor(st[1]);
    im = make_int2((int) fx, (int) fy);
    const double rx = st[0] - fx, ry = st[1] - fy;
    X = (rx * 18446744073709551616.0 >= 18446744073709551615.0) ? ~0ull : __double2ull_rz(rx * 18446744073709551616.0);
    Y = (ry * 18446744073709551616.0 >= 18446744073709551615.0) ? ~0ull : __double2ull_rz(ry * 18446744073709551616.0);
  }
  const int ip = model == 1 ? 2 : 4;
  const double t = st[ip] * 0.15915494309189535;  // phi / (2 pi)
  const double ft = floor(t);
  const double fr = (t - ft) * 4294967296.0;
  const uint32_t ph = fr >= 4294967295.0 ? 0xffffffffu : (uint32_t) fr;
  const float w = (float) st[ip + 1];
  float sp, cp;
  phase_sincos(ph, sp, cp);
  (par ? B.rec1 : B.rec0)[q] = make_uint4((uint32_t) (X >> 32), (uint32_t) (Y >> 32), __float_as_uint(cp),
                                          __float_as_uint(sp));
  (par ? B.aux1 : B.aux0)[q] = make_uint4((uint32_t) X, (uint32_t) Y, ph, __float_as_uint(w));
  B.img[p] = im;
  B.turns[p] = (int) ft;
  if (model == 2) B.vel[q] = make_float2((float) st[2], (float) st[3]);
}

// Download to reference AoS, one thread per original index: gathers the slot
// inv[p]; the block's rows are written as one coalesced chunk.
__global__ void fast_download_kernel(double *__restrict__ x, int n, int s, int model, FastBuffers B)
{
  extern __shared__ double rows[];
  const int p0 = blockIdx.x * blockDim.x;
  const int count = min((int) blockDim.x, n - p0) * s;
  const int p = p0 + threadIdx.x;
  if (p < n)
  {
    const int par = B.ctrl->parity;
    const unsigned q = B.inv[p];
    const uint4 r = (par ? B.rec1 : B.rec0)[q];
    const uint4 a = (par ? B.aux1 : B.aux0)[q];
    const int2 im = B.img[p];
    double *st = rows + s * threadIdx.x;
    st[0] = (double) im.x + (double) join64(r.x, a.x) * 5.421010862427522e-20;
    st[1] = (double) im.y + (double) join64(r.y, a.y) * 5.421010862427522e-20;
    const int ip = model == 1 ? 2 : 4;
    st[ip] = 6.283185307179586 * ((double) B.turns[p] + (double) a.z * 2.3283064365386963e-10);
    st[ip + 1] = (double) __uint_as_float(a.w);
    if (model == 2)
    {
      const float2 v = B.vel[q];
      st[2] = v.x;
      st[3] = v.y;
    }
  }
  __syncthreads();
  rows_from_shared(x + (long) s * p0, rows, count);
}

// ---------------------------------------------------------------- rebuild

// Whether this rebuild covers system `sys`: every system, or those whose own
// trigger fired.  A system left out keeps its slots, cells, tile layouts and
// lists exactly as its last rebuild made them.
__device__ __forceinline__ bool rebuilds_system(const FastBuffers &B, int sys)
{
  return B.ctrl->rebuild != REBUILD_FLAGGED || B.sysctl[sys].rebuild;
}

__global__ void fast_cells_kernel(FastParams P, FastBuffers B)
{
  pdl_enter();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.n || B.ctrl->cells_fresh) return;  // the last step wrote every slot's cell id
  if (!rebuilds_system(B, B.sys_of[q]))
  {
    // sorted by cell since its last rebuild: the stable counting sort leaves it in place
    B.cell_of[q] = B.cell_sorted[q];
    return;
  }
  const int par = B.ctrl->parity;
  const uint4 r = (par ? B.rec1 : B.rec0)[q];
  const uint4 a = (par ? B.aux1 : B.aux0)[q];
  const SysParams *S = B.sys + B.sys_of[q];
  B.cell_of[q] = S->cell0 + cell_of_fix(join64(r.x, a.x), join64(r.y, a.y), S->nc);
}

// New slot q takes the particle of old slot order[q] (cells contiguous,
// ascending old slot inside a cell).  Writes the other rec/aux buffer.
__global__ void fast_permute_kernel(FastParams P, FastBuffers B)
{
  pdl_enter();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.n) return;
  if (!rebuilds_system(B, B.sys_of[q])) return;  // its order is the identity
  const int par = B.ctrl->parity;
  const int src = B.order[q];
  (par ? B.rec0 : B.rec1)[q] = (par ? B.rec1 : B.rec0)[src];
  (par ? B.aux0 : B.aux1)[q] = (par ? B.aux1 : B.aux0)[src];
  const unsigned p = B.pid[src];
  B.pid_tmp[q] = p;
  B.inv[p] = (unsigned) q;
  if (P.model == 2) B.vel_tmp[q] = B.vel[src];
  B.cell_sorted[q] = B.cell_of[src];
}

// A rebuild of every system leaves the permuted records in the other buffer
// (the parity flips); a rebuild of the flagged systems copies theirs back, so
// the systems left out keep their records where they are.
__global__ void fast_copyback_kernel(FastParams P, FastBuffers B)
{
  pdl_enter();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.n) return;
  if (!rebuilds_system(B, B.sys_of[q])) return;
  if (B.ctrl->rebuild == REBUILD_FLAGGED)
  {
    const int par = B.ctrl->parity;
    (par ? B.rec1 : B.rec0)[q] = (par ? B.rec0 : B.rec1)[q];
    (par ? B.aux1 : B.aux0)[q] = (par ? B.aux0 : B.aux1)[q];
  }
  B.pid[q] = B.pid_tmp[q];
  if (P.model == 2) B.vel[q] = B.vel_tmp[q];
}

// The permuted records are current: a rebuild of every system flips the
// buffer parity (the flagged-system form copied its records back).  One
// thread; runs before the tile layouts and list builds, which read them.
__global__ void fast_after_permute_kernel(FastControl *ctrl, int permuted)
{
  pdl_enter();
  if (permuted && ctrl->rebuild != REBUILD_FLAGGED) ctrl->parity ^= 1;
  ctrl->cells_fresh = 0;  // the slots moved
}

// Lists are now current.  The flags are cleared only here, after the tile
// layout and list kernels, so those rebuild the flagged systems alone (with
// the flags cleared before them, every system's layouts and lists were
// rebuilt at each flagged rebuild).  One block.
__global__ void fast_after_rebuild_kernel(FastControl *ctrl, SysControl *sysctl, int nsys)
{
  pdl_enter();
  for (int r = threadIdx.x; r < nsys; r += blockDim.x) sysctl[r].rebuild = 0;
  if (threadIdx.x == 0)
  {
    ctrl->rebuild = REBUILD_NONE;
    ctrl->rebuilds += 1;
  }
}

// ---------------------------------------------------------------- tiles
//
// A tile is a run of whole cells of one row of a system's rebuild grid; one
// CTA steps the particles of a tile.  A row holds ceil(nc / tile_cells) tiles.
// With Verlet lists they split the row's particles into runs of nearly equal
// count (boundaries at cell edges), so a tile of about 120 particles fills
// its 128 threads whatever the local density, where runs of equal width leave
// Poisson counts above 128 to a second pass of a few threads (36-cell tiles
// at N = 4,194,304: 0.1963 -> 0.1882 ms per launch, same bits); the layout is
// computed once per rebuild.  Cell lists lay their tiles out every step and
// keep runs of tile_cells cells: the binary searches of the equal-count
// boundaries, and widths beyond the run table, cost more there than the fuller
// warps gain (measured 0.622 -> 0.645 ms per step at N = 4,194,304).  Slots are
// sorted by cell, so the tile's particles are one slot range and the records
// of its 3 x (width + 2) neighbour cells are at most six slot segments (three
// rows, each split in two where the periodic x-wrap crosses the row end).
// The CTA stages those segments into shared memory with TMA bulk copies; the
// Verlet list of a particle in a staged tile stores shared-memory indices
// directly.

constexpr int kTileCellsDefault = 32;  // cells per tile unless tuned
constexpr int kTileCap = 512;     // staged neighbour records per CTA (2 x 8 KiB)
constexpr int kTileThreads = 128;
// Resident CTAs per SM the Stochastic Euler tile kernels are compiled for.
// Cell lists: 14 (32 registers, some spilled; the 512-system sweep step ran
// 1.197 / 1.283 / 1.354 ms at 14 / 12 / 10).  Verlet lists: 10 (48 registers, 4 to 16 bytes spilled); the 512-system
// sweep at 36-cell tiles ran 0.684 / 0.623 / 0.553 / 0.573 ms per step at
// 14 / 12 / 10 / 9.
#ifndef SPSS_SE_TILE_BLOCKS
#define SPSS_SE_TILE_BLOCKS 14
#endif
#ifndef SPSS_SE_VERLET_TILE_BLOCKS
#define SPSS_SE_VERLET_TILE_BLOCKS 10
#endif
constexpr long long kWaitCycles = 1ll << 31;  // about one second at the SM clock

struct TileLayout
{
  int p_begin, p_end;  // slots of the tile's own particles
  int nseg, total;     // staged segments (ascending slot order) and records
  int start[6], len[6], base[6];
  int staged;          // the neighbourhood fits kTileCap records
  int row, col0, ncols;  // the tile's cells: row `row`, columns col0 .. col0 + ncols - 1
};

// Cell-list stencil of one cell of a staged tile: for each stencil row (dy =
// -1, 0, 1) the staged records of the three cells (cx - 1, cx, cx + 1, wrapped)
// as at most three contiguous runs of staged indices, in the reference's
// stencil order (ParticleSystemFirstOrder.cpp:47-52).
constexpr int kRunCells = 64;  // widest tile with a run table
struct StencilRuns
{
  short s[3][3], e[3][3];  // [dy + 1][piece]
};

__host__ __device__ __forceinline__ int tiles_per_row(int nc, int tc)
{
  return (nc + tc - 1) / tc;
}

// Equal-count tiles: the row's particles split into `nbx` runs of whole
// cells, boundary k at the first cell edge where the row's running count
// reaches k * (row count) / nbx.
__device__ __forceinline__ int row_target(const int *__restrict__ ro, int nc, int k, int nbx)
{
  return ro[0] + (int) ((long long) (ro[nc] - ro[0]) * k / nbx);
}

__device__ __forceinline__ int first_cell_reaching(const int *__restrict__ ro, int nc, int target)
{
  int lo = 0, hi = nc;  // ro[hi] >= target always
  while (lo < hi)
  {
    const int mid = (lo + hi) >> 1;
    if (ro[mid] >= target) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// Deterministic layout of tile t of a system (cell offsets `off` of that
// system's grid; the list build and the step compute the same).
__device__ void tile_layout(int t, int nc, int tc, const int *__restrict__ off, bool equal_count, TileLayout &L)
{
  const int nbx = tiles_per_row(nc, tc);
  const int cy = t / nbx, bx = t - cy * nbx;
  const int *ro = off + cy * nc;
  int cx_lo, cx_hi;
  if (equal_count)
  {
    cx_lo = first_cell_reaching(ro, nc, row_target(ro, nc, bx, nbx));
    cx_hi = bx + 1 == nbx ? nc : first_cell_reaching(ro, nc, row_target(ro, nc, bx + 1, nbx));
  } else
  {
    cx_lo = bx * tc;
    cx_hi = min(nc, cx_lo + tc);
  }
  L.p_begin = off[cy * nc + cx_lo];
  L.p_end = off[cy * nc + cx_hi];
  L.row = cy;
  L.col0 = cx_lo;
  L.ncols = cx_hi - cx_lo;
  L.nseg = 0;
  L.total = 0;
  L.staged = 0;
  if (nc < 3) return;  // rows would repeat in the stencil
  int st[6], en[6], ns = 0;
  const bool whole_row = (cx_hi - cx_lo + 2) >= nc;
  for (int dy = -1; dy <= 1; ++dy)
  {
    const int row = wrap_cell(cy + dy, nc) * nc;
    if (whole_row)
    {
      st[ns] = off[row];
      en[ns++] = off[row + nc];
    } else if (cx_lo == 0)
    {
      st[ns] = off[row];  // cells 0 .. cx_hi
      en[ns++] = off[row + cx_hi + 1];
      st[ns] = off[row + nc - 1];  // left neighbour wraps to the last cell
      en[ns++] = off[row + nc];
    } else if (cx_hi == nc)
    {
      st[ns] = off[row];  // right neighbour wraps to the first cell
      en[ns++] = off[row + 1];
      st[ns] = off[row + cx_lo - 1];
      en[ns++] = off[row + nc];
    } else
    {
      st[ns] = off[row + cx_lo - 1];
      en[ns++] = off[row + cx_hi + 1];
    }
  }
  for (int a = 1; a < ns; ++a)
  {
    const int s0 = st[a], e0 = en[a];
    int b = a - 1;
    while (b >= 0 && st[b] > s0)
    {
      st[b + 1] = st[b];
      en[b + 1] = en[b];
      --b;
    }
    st[b + 1] = s0;
    en[b + 1] = e0;
  }
  for (int a = 0; a < ns; ++a)
  {
    if (en[a] <= st[a]) continue;
    L.start[L.nseg] = st[a];
    L.len[L.nseg] = en[a] - st[a];
    L.base[L.nseg] = L.total;
    L.total += en[a] - st[a];
    ++L.nseg;
  }
  L.staged = L.total <= kTileCap;
}

// Layout of every tile of every system, once per rebuild.
__global__ void fast_tile_layout_kernel(FastParams P, FastBuffers B)
{
  pdl_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.ntiles) return;
  if (!rebuilds_system(B, B.tile_sys[t])) return;
  const SysParams *S = B.sys + B.tile_sys[t];
  TileLayout L;
  tile_layout(t - S->tile0, S->nc, P.tile_cells, B.cell_off + S->cell0, P.kind == KIND_VERLET, L);
  reinterpret_cast<TileLayout *>(B.tiles)[t] = L;
}

// Tile-major Verlet lists: tile t keeps rows m = 0 .. cap-1 of its particles
// contiguously, row stride round_up8(particles of the tile) entries, starting
// at cap * round_up8(p_begin + 16 t) (16-byte aligned, never overlapping the
// next tile); a tile's list rows are thus one block a bulk copy can stage.
__device__ __forceinline__ long tile_list_base(int cap, int t, int p_begin)
{
  return (long) cap * (long) ((p_begin + 16 * t + 7) & ~7);
}

__device__ __forceinline__ int tile_list_stride(int p_begin, int p_end)
{
  return (p_end - p_begin + 7) & ~7;
}

constexpr int kListCap = 4096;  // staged list entries per CTA (8 KiB)

// Shared-memory index of slot j inside the staged segments (-1: not staged).
__device__ __forceinline__ int staged_index(const TileLayout &L, int j)
{
  for (int k = 0; k < L.nseg; ++k)
    if (j >= L.start[k] && j < L.start[k] + L.len[k]) return L.base[k] + (j - L.start[k]);
  return -1;
}

// Slot of a staged index (rare path: the guard band needs the slot's low words).
__device__ __forceinline__ int staged_slot(const TileLayout &L, int idx)
{
  for (int k = 0; k < L.nseg; ++k)
    if (idx >= L.base[k] && idx < L.base[k] + L.len[k]) return L.start[k] + (idx - L.base[k]);
  return 0;
}

// Run table and per-particle cell column of a staged tile (all threads of the
// CTA; cell offsets `coff` of the tile's system).  Returns through `self_base`
// the shift from a slot of the tile to its staged index.
__device__ __forceinline__ void build_runs(const TileLayout &L, const int *__restrict__ coff, int nc,
                                           StencilRuns *runs, unsigned char *col_of, int *self_base, int *error)
{
  for (int w = threadIdx.x; w < 3 * L.ncols; w += blockDim.x)
  {
    const int k = w / 3, dy = w - 3 * k - 1;
    const int cx = L.col0 + k;
    const int row = wrap_cell(L.row + dy, nc) * nc;
    const int cells[3] = {wrap_cell(cx - 1, nc), cx, wrap_cell(cx + 1, nc)};
    short ps[3] = {0, 0, 0}, pe[3] = {0, 0, 0};
    int np = 0;
    for (int u = 0; u < 3; ++u)
    {
      const int b = coff[row + cells[u]], e = coff[row + cells[u] + 1];
      if (e <= b) continue;
      const int i0 = staged_index(L, b);
      if (i0 < 0)
      {
        atomicOr(error, 4);  // a stencil cell outside the staged segments (the layout rules this out)
        continue;
      }
      if (np > 0 && pe[np - 1] == i0)
      {
        pe[np - 1] = (short) (i0 + (e - b));
      } else
      {
        ps[np] = (short) i0;
        pe[np] = (short) (i0 + (e - b));
        ++np;
      }
    }
    for (int u = 0; u < 3; ++u)
    {
      runs[k].s[dy + 1][u] = ps[u];
      runs[k].e[dy + 1][u] = pe[u];
    }
    if (dy == 0)
    {
      const int rb = L.row * nc;
      for (int q = coff[rb + cx]; q < coff[rb + cx + 1]; ++q) col_of[q - L.p_begin] = (unsigned char) k;
    }
  }
  if (threadIdx.x == 0)
  {
    for (int k = 0; k < L.nseg; ++k)
      if (L.p_begin >= L.start[k] && L.p_begin < L.start[k] + L.len[k]) *self_base = L.base[k] - L.start[k];
  }
}

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return (uint32_t) __cvta_generic_to_shared(p);
}

// Verlet lists from the 3x3 stencil of the rebuild grid (ParticleSystemFirstOrder.cpp:536-589):
// pairs with r <= r_max (conservatively widened by the guard band; an entry
// beyond r_max can never come within rho before the next rebuild).  Entry m of
// slot q at vl[m * n + q] (16 bits): the neighbour's shared-memory index when
// q's tile is staged, else the offset j - q.  A count of -1 marks a list
// longer than the capacity or an offset beyond 16 bits; the step then scans
// the stencil of the rebuild-time cell instead.  This per-slot form (global
// gathers) serves the tiles whose neighbourhood is not staged; the staged
// tiles build in fast_verlet_tile_build_kernel.
__device__ void verlet_build_slot(const FastParams &P, const FastBuffers &B, int q, int t)
{
  const int par = B.ctrl->parity;
  const uint4 *rec = par ? B.rec1 : B.rec0;
  const uint4 ri = rec[q];
  const SysParams *S = B.sys + B.sys_of[q];
  const int nc = S->nc;
  const float rmax2_f = S->rmax2_f;
  const int *coff = B.cell_off + S->cell0;
  const int c = B.cell_sorted[q] - S->cell0;
  const int cx = c % nc, cy = c / nc;
  const TileLayout L = reinterpret_cast<const TileLayout *>(B.tiles)[t];
  int cnt = 0;
  bool far = false;
  const int stride = tile_list_stride(L.p_begin, L.p_end);
  short *lp = B.vl + tile_list_base(P.cap, t, L.p_begin) + (q - L.p_begin);
  for (int sy = -1; sy <= 1; ++sy)
  {
    const int jy = wrap_cell(cy + sy, nc);
    for (int sx = -1; sx <= 1; ++sx)
    {
      const int jc = jy * nc + wrap_cell(cx + sx, nc);
      const int e = coff[jc + 1];
      for (int j = coff[jc]; j < e; ++j)
      {
        if (j == q) continue;
        const uint4 rj = __ldg(&rec[j]);
        const float dx = (float) (int) (rj.x - ri.x);
        const float dy = (float) (int) (rj.y - ri.y);
        if (fmaf(dx, dx, dy * dy) <= rmax2_f)
        {
          int entry;
          if (L.staged)
          {
            entry = staged_index(L, j);
            if (entry < 0) far = true;
          } else
          {
            entry = j - q;
            if (entry < -32768 || entry > 32767) far = true;
          }
          if (cnt < P.cap)
          {
            *lp = (short) entry;
            lp += stride;
          }
          ++cnt;
        }
      }
    }
  }
  if (cnt > P.cap) atomicMax(&B.ctrl->overflow, cnt);
  atomicMax(&B.tile_maxcnt[t], min(cnt, P.cap));
  B.vl_cnt[q] = (cnt > P.cap || far) ? -1 : cnt;
}

// ---------------------------------------------------------------- step

// Neighbour sums of slot q from global memory (per-slot kernel, and tiles
// that do not fit shared memory): the Verlet list holds slot offsets.
template<int KIND, bool OMEGA>
__device__ __forceinline__ void gather_sums(const FastParams &P, const FastBuffers &B, const uint4 *__restrict__ rec,
                                            const uint4 *__restrict__ aux, int q, int cnt, const short *lp, int stride,
                                            const uint4 &ri, uint64_t Xi, uint64_t Yi, Acc &a)
{
  if (KIND == KIND_VERLET)
  {
    if (cnt >= 0)
    {
      const long n = stride;
      int m = 0;
      for (; m + 4 <= cnt; m += 4)
      {
        const int j[4] = {q + (int) lp[0], q + (int) lp[n], q + (int) lp[2 * n], q + (int) lp[3 * n]};
        lp += 4 * n;
        candidates4<OMEGA, KIND == KIND_CELLS>(P, ri, Xi, Yi, rec, aux, j, a);
      }
      for (; m < cnt; ++m)
      {
        const int j = q + (int) lp[0];
        lp += n;
        candidate<OMEGA, KIND == KIND_CELLS>(P, ri, Xi, Yi, rec, aux, j, a);
      }
      return;
    }
    // list unusable: the stencil of the rebuild-time cell holds every particle
    // the list would (displacements since the rebuild < skin / 2)
  }
  if (KIND == KIND_ALL_PAIRS)
  {
    const int end = P.first + P.sub_n;
    for (int j = P.first; j < end; ++j)
      if (j != q) candidate<OMEGA, KIND == KIND_CELLS>(P, ri, Xi, Yi, rec, aux, j, a);
    return;
  }
  const int *coff = B.cell_off + P.cell0;
  const int c = B.cell_sorted[q] - P.cell0;
  const int cx = c % P.nc, cy = c / P.nc;
  // stencil in the reference's order (-1,-1),(0,-1),(1,-1),(-1,0),... (ParticleSystemFirstOrder.cpp:47-52)
  for (int sy = -1; sy <= 1; ++sy)
  {
    const int jy = wrap_cell(cy + sy, P.nc);
    for (int sx = -1; sx <= 1; ++sx)
    {
      const int jc = jy * P.nc + wrap_cell(cx + sx, P.nc);
      const int e = coff[jc + 1];
      for (int j = coff[jc]; j < e; ++j)
        if (j != q) candidate<OMEGA, KIND == KIND_CELLS>(P, ri, Xi, Yi, rec, aux, j, a);
    }
  }
}

// The FP64 cutoff decision for a staged candidate inside the guard band when
// the aux words are not staged (steppers that need no neighbour omega): the
// low position words come from global memory at the candidate's slot.
__device__ __forceinline__ bool exact_within_slot_inline(const TileLayout &L, const uint4 *__restrict__ aux, int idx,
                                                        uint32_t xh, uint32_t yh, uint64_t Xi, uint64_t Yi,
                                                        double rho2)
{
  const uint2 l = __ldg(reinterpret_cast<const uint2 *>(&aux[staged_slot(L, idx)]));
  return exact_within_inline(xh, yh, l.x, l.y, Xi, Yi, rho2);
}

__device__ __noinline__ bool exact_within_slot(const TileLayout &L, const uint4 *__restrict__ aux, int idx,
                                               uint32_t xh, uint32_t yh, uint64_t Xi, uint64_t Yi, double rho2)
{
  return exact_within_slot_inline(L, aux, idx, xh, yh, Xi, Yi, rho2);
}

// One staged candidate: the record comes from shared memory; the guard band
// (rare) takes the slot's low position words from the staged aux words (SRK,
// which stages them for the neighbours' omega) or from global memory (SE).
template<bool OMEGA, bool OUTLINE = true>
__device__ __forceinline__ void candidate_staged(const FastParams &P, const uint4 &ri, uint64_t Xi, uint64_t Yi,
                                                 const uint4 *srec, const uint4 *saux, const TileLayout &L,
                                                 const uint4 *__restrict__ aux, int idx, Acc &a)
{
  const uint4 rj = srec[idx];
  // the omega word is loaded with the record, before the range test, so the
  // two shared-memory loads overlap instead of forming a dependent chain
  const float wj = OMEGA ? __uint_as_float(saux[idx].w) : 0.0f;
  const float dx = (float) (int) (rj.x - ri.x);
  const float dy = (float) (int) (rj.y - ri.y);
  const float d2 = fmaf(dx, dx, dy * dy);
  bool in = d2 <= P.rho2_f;
  if (fabsf(d2 - P.rho2_f) <= P.band_f)
  {
    if (OMEGA)
    {
      const uint4 l = saux[idx];
      in = OUTLINE ? exact_within(rj.x, rj.y, l.x, l.y, Xi, Yi, P.rho2_d)
                   : exact_within_inline(rj.x, rj.y, l.x, l.y, Xi, Yi, P.rho2_d);
    } else
    {
      in = OUTLINE ? exact_within_slot(L, aux, idx, rj.x, rj.y, Xi, Yi, P.rho2_d)
                   : exact_within_slot_inline(L, aux, idx, rj.x, rj.y, Xi, Yi, P.rho2_d);
    }
  }
  if (in) accumulate(a, rj, wj);
}

// Neighbour sums of slot q from the tile's staged records.
template<int KIND, bool OMEGA>
__device__ __forceinline__ void gather_sums_staged(const FastParams &P, const FastBuffers &B, const uint4 *srec,
                                                   const uint4 *saux, const TileLayout &L,
                                                   const uint4 *__restrict__ rec, const uint4 *__restrict__ aux, int q,
                                                   int cnt, const short *lp, int stride, const uint4 &ri, uint64_t Xi,
                                                   uint64_t Yi, Acc &a, const StencilRuns *runs,
                                                   const unsigned char *col_of, int self_base)
{
  if (KIND == KIND_CELLS && runs)
  {
    // cell list from the tile's run table: three rows of contiguous staged
    // records.  The guard-band decision is inline for Stochastic Euler (no
    // call in the loop: the batched 512-system sweep step 1.319 -> 1.197 ms,
    // N = 65,536 0.0638 -> 0.0622 ms, fewer spills at 32 registers) and out of
    // line for SRK, whose larger kernel ran 0.7 % slower with it inline.
    const StencilRuns &R = runs[col_of[q - L.p_begin]];
    const int self = q + self_base;
#pragma unroll 1
    for (int r = 0; r < 3; ++r)
#pragma unroll 1
      for (int u = 0; u < 3; ++u)
      {
        const int e = R.e[r][u];
        for (int idx = R.s[r][u]; idx < e; ++idx)
          if (idx != self) candidate_staged<OMEGA, OMEGA>(P, ri, Xi, Yi, srec, saux, L, aux, idx, a);
      }
    return;
  }
  if (KIND == KIND_VERLET && cnt >= 0)
  {
    const long n = stride;
    int m = 0;
    for (; m + 4 <= cnt; m += 4)
    {
      // four candidates as one group: entries, records and omega words loaded
      // together, four FP32 distances, one guard-band test for the group (a
      // group with a candidate inside the band is redone one by one with the
      // FP64 decision there), so the common path has no branch between loads
      const int i[4] = {lp[0], lp[n], lp[2 * n], lp[3 * n]};
      lp += 4 * n;
      uint4 r[4];
      float w[4], d2[4];
#pragma unroll
      for (int k = 0; k < 4; ++k)
      {
        r[k] = srec[i[k]];
        w[k] = OMEGA ? __uint_as_float(saux[i[k]].w) : 0.0f;
      }
      bool band = false;
#pragma unroll
      for (int k = 0; k < 4; ++k)
      {
        const float dx = (float) (int) (r[k].x - ri.x);
        const float dy = (float) (int) (r[k].y - ri.y);
        d2[k] = fmaf(dx, dx, dy * dy);
        band |= fabsf(d2[k] - P.rho2_f) <= P.band_f;
      }
      if (!band)
      {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (d2[k] <= P.rho2_f) accumulate(a, r[k], w[k]);
      } else
      {
#pragma unroll 1
        for (int k = 0; k < 4; ++k) candidate_staged<OMEGA, true>(P, ri, Xi, Yi, srec, saux, L, aux, i[k], a);
      }
    }
    for (; m < cnt; ++m)
    {
      candidate_staged<OMEGA, false>(P, ri, Xi, Yi, srec, saux, L, aux, lp[0], a);
      lp += n;
    }
    return;
  }
  // cell list, or a Verlet list that did not fit: scan the stencil of the
  // (rebuild-time) cell; each stencil cell is one contiguous staged range
  const int *coff = B.cell_off + P.cell0;
  const int c = B.cell_sorted[q] - P.cell0;
  const int cx = c % P.nc, cy = c / P.nc;
  for (int sy = -1; sy <= 1; ++sy)
  {
    const int jy = wrap_cell(cy + sy, P.nc);
    for (int sx = -1; sx <= 1; ++sx)
    {
      const int jc = jy * P.nc + wrap_cell(cx + sx, P.nc);
      const int b = coff[jc], e = coff[jc + 1];
      if (e <= b) continue;
      const int i0 = staged_index(L, b);
      if (i0 < 0 || i0 + (e - b) > L.total)
      {
        // not inside the staged segments (cannot happen for a cell of this tile's stencil)
        for (int j = b; j < e; ++j)
          if (j != q) candidate<OMEGA, KIND == KIND_CELLS>(P, ri, Xi, Yi, rec, aux, j, a);
        continue;
      }
      const int self = q - b;
      for (int u = 0; u < e - b; ++u)
        if (u != self) candidate_staged<OMEGA, KIND == KIND_CELLS>(P, ri, Xi, Yi, srec, saux, L, aux, i0 + u, a);
    }
  }
}

// Exactly the normals the stepper consumes, in the reference's draw order.
template<int MODEL, int STEPPER>
__device__ __forceinline__ void draw_noise(const FastParams &P, unsigned long long step, unsigned p, float z[6])
{
  constexpr int kNeed = MODEL == 1 ? (STEPPER == 1 ? 1 : 2) : (STEPPER == 1 ? 3 : 6);
  p -= (unsigned) P.first;  // index of the particle within its system
  // philox_block(seed, replica, step; p, block 0) with the round keys from the parameters
  const uint4 u = philox_keyed(make_uint4(p, (uint32_t) step, (uint32_t) (step >> 32), P.replica << 8), P.kx, P.ky);
  if (kNeed > 4)
  {
    box_muller6_f32(u, z);  // six normals from the one block
    return;
  }
  box_muller_f32(u.x, u.y, z[0], z[1]);
  if (kNeed > 2) box_muller_f32(u.z, u.w, z[2], z[3]);
}

// Torque derivative f_w and (SRK) complementary force C from the neighbour
// sums.  Every rounding step is spelled out (fmaf, __fmul_rn, __fadd_rn): the
// compiler cannot contract or reassociate, so each instantiation (one system
// or a batch) rounds identically.
template<int STEPPER>
__device__ __forceinline__ void sums_forces(const FastParams &P, const Acc &a, float cphi, float sphi, float wi,
                                            float &f_w, float &C)
{
  // sum sin(phi_j - phi_i - alpha) and sum (omega_j - omega_i) cos(phi_j - phi_i - alpha)
  f_w = 0.0f;  // SE/SRK zero-fill the derivative: an isolated particle keeps 0
  C = 0.0f;
  if (a.card > 0)
  {
    const float inv = 1.0f / (float) a.card;
    const float S = fmaf(cphi, a.ss, -__fmul_rn(sphi, a.sc));  // sum sin(phi_j - phi_i)
    const float K = fmaf(cphi, a.sc, __fmul_rn(sphi, a.ss));   // sum cos(phi_j - phi_i)
    f_w = fmaf(-P.xi_phi, wi, __fmul_rn(__fmul_rn(P.sigma, fmaf(P.ca, S, -__fmul_rn(P.sa, K))), inv));
    if (STEPPER == 2)
    {
      const float WS = fmaf(cphi, a.ws, -__fmul_rn(sphi, a.wc));  // sum omega_j sin(phi_j - phi_i)
      const float WK = fmaf(cphi, a.wc, __fmul_rn(sphi, a.ws));   // sum omega_j cos(phi_j - phi_i)
      C = __fmul_rn(__fmul_rn(P.sigma, inv), __fsub_rn(fmaf(P.ca, WK, __fmul_rn(P.sa, WS)),
                                                       __fmul_rn(wi, fmaf(P.ca, K, __fmul_rn(P.sa, S)))));
    }
  }
}

template<int MODEL, int STEPPER>
__device__ __forceinline__ float advance_particle(const FastParams &P, const FastBuffers &B, int q, const uint4 &ri,
                                                  const uint4 &ai, float2 v, float f_w, float C, const float z[6],
                                                  uint4 *rout, uint4 *aout, int &err, int *cell_out = nullptr);

// Derivative from the neighbour sums, SE or SRK update in fixed point, new
// record.  Returns |dr|^2 of the step.
template<int MODEL, int STEPPER>
__device__ __forceinline__ float update_particle(const FastParams &P, const FastBuffers &B, int q, const uint4 &ri,
                                                 const uint4 &ai, float2 v, const Acc &a, const float z[6],
                                                 uint4 *rout, uint4 *aout, int &err, int *cell_out = nullptr)
{
  float f_w, C;
  sums_forces<STEPPER>(P, a, __uint_as_float(ri.z), __uint_as_float(ri.w), __uint_as_float(ai.w), f_w, C);
  return advance_particle<MODEL, STEPPER>(P, B, q, ri, ai, v, f_w, C, z, rout, aout, err, cell_out);
}

// SE or SRK update in fixed point from the forces, new record.  Returns
// |dr|^2 of the step.  `cell_out` (cell-list steps): the new position's cell
// id at the slot, which the next step's cell-list rebuild then need not
// recompute.
template<int MODEL, int STEPPER>
__device__ __forceinline__ float advance_particle(const FastParams &P, const FastBuffers &B, int q, const uint4 &ri,
                                                  const uint4 &ai, float2 v, float f_w, float C, const float z[6],
                                                  uint4 *rout, uint4 *aout, int &err, int *cell_out)
{
  const uint64_t Xi = join64(ri.x, ai.x), Yi = join64(ri.y, ai.y);
  const float cphi = __uint_as_float(ri.z), sphi = __uint_as_float(ri.w);
  const float wi = __uint_as_float(ai.w);
  const float dt = P.dt;
  float ddx, ddy, dphi, dw;
  if (MODEL == 1)
  {
    const float fx = __fmul_rn(P.v0, cphi), fy = __fmul_rn(P.v0, sphi), fp = wi;
    if (STEPPER == 1)
    {
      // StochasticEulerStepperPtr.hpp:58-66
      ddx = __fmul_rn(fx, dt);
      ddy = __fmul_rn(fy, dt);
      dphi = __fmul_rn(fp, dt);
      dw = fmaf(f_w, dt, __fmul_rn(P.b_phi, __fmul_rn(P.sqdt, z[0])));
    } else
    {
      // StochasticRungeKuttaStepperPtr.hpp:54-70
      const float dW = __fmul_rn(z[0], P.sqdt);
      const float dZ = __fmul_rn(P.half_dt15, fmaf(P.inv_sqrt3, z[1], z[0]));
      ddx = fmaf(fx, dt, -__fmul_rn(__fmul_rn(fp, fy), P.half_dt2));
      ddy = fmaf(fy, dt, __fmul_rn(__fmul_rn(fp, fx), P.half_dt2));
      dphi = fmaf(fp, dt, fmaf(f_w, P.half_dt2, __fmul_rn(P.b_phi, dZ)));
      dw = fmaf(f_w, dt, fmaf(fmaf(-P.xi, f_w, C), P.half_dt2, __fmul_rn(P.b_phi, fmaf(-P.xi, dZ, dW))));
    }
  } else
  {
    const float fvx = fmaf(-P.xi_r, v.x, __fmul_rn(P.v0, cphi));
    const float fvy = fmaf(-P.xi_r, v.y, __fmul_rn(P.v0, sphi));
    float dvx, dvy;
    if (STEPPER == 1)
    {
      // StochasticEulerStepper.hpp:44-50 with AddNoise (ParticleSystemSecondOrder.cpp:447-449)
      ddx = __fmul_rn(dt, v.x);
      ddy = __fmul_rn(dt, v.y);
      dvx = fmaf(dt, fvx, __fmul_rn(P.sqdt, __fmul_rn(P.b_r, z[0])));
      dvy = fmaf(dt, fvy, __fmul_rn(P.sqdt, __fmul_rn(P.b_r, z[1])));
      dphi = __fmul_rn(dt, wi);
      dw = fmaf(dt, f_w, __fmul_rn(P.sqdt, __fmul_rn(P.b_phi, z[2])));
    } else
    {
      // second-order strong order 1.5 Taylor scheme (no reference code)
      const float dWx = __fmul_rn(z[0], P.sqdt), dZx = __fmul_rn(P.half_dt15, fmaf(P.inv_sqrt3, z[1], z[0]));
      const float dWy = __fmul_rn(z[2], P.sqdt), dZy = __fmul_rn(P.half_dt15, fmaf(P.inv_sqrt3, z[3], z[2]));
      const float dWw = __fmul_rn(z[4], P.sqdt), dZw = __fmul_rn(P.half_dt15, fmaf(P.inv_sqrt3, z[5], z[4]));
      ddx = fmaf(v.x, dt, fmaf(fvx, P.half_dt2, __fmul_rn(P.b_r, dZx)));
      ddy = fmaf(v.y, dt, fmaf(fvy, P.half_dt2, __fmul_rn(P.b_r, dZy)));
      dvx = fmaf(fvx, dt, fmaf(fmaf(-P.xi_r, fvx, -__fmul_rn(__fmul_rn(P.v0, sphi), wi)), P.half_dt2,
                               __fmul_rn(P.b_r, fmaf(-P.xi_r, dZx, dWx))));
      dvy = fmaf(fvy, dt, fmaf(fmaf(-P.xi_r, fvy, __fmul_rn(__fmul_rn(P.v0, cphi), wi)), P.half_dt2,
                               __fmul_rn(P.b_r, fmaf(-P.xi_r, dZy, dWy))));
      dphi = fmaf(wi, dt, fmaf(f_w, P.half_dt2, __fmul_rn(P.b_phi, dZw)));
      dw = fmaf(f_w, dt, fmaf(fmaf(-P.xi_phi, f_w, C), P.half_dt2, __fmul_rn(P.b_phi, fmaf(-P.xi_phi, dZw, dWw))));
    }
    B.vel[q] = make_float2(__fadd_rn(v.x, dvx), __fadd_rn(v.y, dvy));
  }
  int cx, cy, ct;
  const uint64_t Xn = advance(Xi, fix64_of(ddx, err), cx);
  const uint64_t Yn = advance(Yi, fix64_of(ddy, err), cy);
  const uint32_t Pn = advance_phase(ai.z, dphi, ct, err);
  float sn, cn;
  phase_sincos(Pn, sn, cn);
  rout[q] = make_uint4((uint32_t) (Xn >> 32), (uint32_t) (Yn >> 32), __float_as_uint(cn), __float_as_uint(sn));
  aout[q] = make_uint4((uint32_t) Xn, (uint32_t) Yn, Pn, __float_as_uint(__fadd_rn(wi, dw)));
  if (cell_out) cell_out[q] = P.cell0 + cell_of_fix(Xn, Yn, P.nc);
  // box crossings and phase turns are rare: read-modify-write only then (the
  // counts are kept by original index, so the slot re-sort never moves them)
  if (cx | cy | ct)
  {
    const unsigned p = B.pid[q];
    if (cx | cy)
    {
      const int2 im = B.img[p];
      B.img[p] = make_int2(im.x + cx, im.y + cy);
    }
    if (ct) B.turns[p] += ct;
  }
  return fmaf(ddx, ddx, __fmul_rn(ddy, ddy));
}

// max |dr|^2 of each system for its Verlet trigger: a warp whose lanes all
// belong to one system reduces first and issues one atomic, and only when it
// can raise the maximum already stored (no block barrier).
__device__ __forceinline__ void raise_max(SysControl *sc, float d2)
{
  const unsigned bits = __float_as_uint(d2);
  if (bits > *(volatile unsigned *) &sc->max2_bits) atomicMax(&sc->max2_bits, bits);
}

__device__ __forceinline__ void publish_max(FastControl *ctrl, SysControl *sysctl, int sys, float d2max, int err)
{
  const int sys0 = __shfl_sync(0xffffffffu, sys, 0);
  if (__all_sync(0xffffffffu, sys == sys0))
  {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) d2max = fmaxf(d2max, __shfl_xor_sync(0xffffffffu, d2max, off));
    if ((threadIdx.x & 31) == 0) raise_max(sysctl + sys0, d2max);
  } else
  {
    raise_max(sysctl + sys, d2max);
  }
  err = __any_sync(0xffffffffu, err);
  if ((threadIdx.x & 31) == 0 && err) atomicOr(&ctrl->error, 1);
}

// One SE or SRK step of one particle per thread, neighbours gathered from
// global memory (all pairs; also usable for every kind).
template<int MODEL, int STEPPER, int KIND, bool MULTI>
__global__ void __launch_bounds__(kTB, 4) fast_step_kernel(FastParams P, FastBuffers B)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  FastControl *ctrl = B.ctrl;
  const int par = ctrl->parity;
  const uint4 *rin = par ? B.rec1 : B.rec0;
  const uint4 *ain = par ? B.aux1 : B.aux0;
  uint4 *rout = par ? B.rec0 : B.rec1;
  uint4 *aout = par ? B.aux0 : B.aux1;
  float d2max = 0.0f;
  int err = 0;
  int sys = 0;
  if (q < P.n)
  {
    sys = MULTI ? B.sys_of[q] : 0;
    const FastParams Q = MULTI ? with_system(P, B.sys[sys]) : P;
    const unsigned p = B.pid[q];
    const uint4 ri = rin[q];
    const uint4 ai = ain[q];
    const float2 v = MODEL == 2 ? B.vel[q] : make_float2(0.f, 0.f);
    float z[6];
    draw_noise<MODEL, STEPPER>(Q, ctrl->step, p, z);  // overlaps the loads above
    Acc a{0.f, 0.f, 0.f, 0.f, 0};
    gather_sums<KIND, STEPPER == 2>(Q, B, rin, ain, q, KIND == KIND_VERLET ? -1 : 0, nullptr, 0, ri,
                                    join64(ri.x, ai.x), join64(ri.y, ai.y), a);
    d2max = update_particle<MODEL, STEPPER>(Q, B, q, ri, ai, v, a, z, rout, aout, err);
  }
  publish_max(ctrl, B.sysctl, sys, d2max, err);
}

// Bounded wait for phase `phase` of an mbarrier (about one second).
__device__ __forceinline__ uint32_t wait_phase(uint32_t mb, uint32_t phase)
{
  uint32_t done = 0;
  const long long t0 = clock64();
  while (!done && clock64() - t0 < kWaitCycles)
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(mb), "r"(phase)
                 : "memory");
  return done;
}

// A particle's own words, loaded from global memory at its slot.
struct OwnParticle
{
  unsigned p;  // original index (noise counter)
  uint4 r, a;  // record and aux words
  int cnt;     // Verlet list length
  float2 v;    // velocity (second order)
};

template<int MODEL, int KIND>
__device__ __forceinline__ OwnParticle load_own(const FastBuffers &B, const uint4 *rin, const uint4 *ain, int q)
{
  OwnParticle o;
  o.p = B.pid[q];
  o.r = rin[q];
  o.a = ain[q];
  o.cnt = KIND == KIND_VERLET ? B.vl_cnt[q] : 0;
  o.v = MODEL == 2 ? B.vel[q] : make_float2(0.f, 0.f);
  return o;
}

// The particles of one tile, one per thread; `o` holds the thread's first
// particle, loaded before the wait for the tile's bulk copies.  The noise is
// drawn after the neighbour walk (fewer registers live across the walk).
template<int MODEL, int STEPPER, int KIND>
__device__ __forceinline__ void step_tile(const FastParams &Q, const FastBuffers &B, const TileLayout &L,
                                          OwnParticle o, const uint4 *srec, const uint4 *saux, const short *slist,
                                          const short *glist, int list_staged, int list_stride, bool staged,
                                          const uint4 *rin, const uint4 *ain, uint4 *rout, uint4 *aout, float &d2max,
                                          int &err, const StencilRuns *runs, const unsigned char *col_of,
                                          int self_base)
{
  const int q0 = L.p_begin + threadIdx.x;
  for (int q = q0; q < L.p_end; q += blockDim.x)
  {
    if (q != q0) o = load_own<MODEL, KIND>(B, rin, ain, q);
    Acc a{0.f, 0.f, 0.f, 0.f, 0};
    const uint64_t Xi = join64(o.r.x, o.a.x), Yi = join64(o.r.y, o.a.y);
    const int i = q - L.p_begin;
    const short *lp = KIND == KIND_VERLET ? (list_staged ? slist + i : glist + i) : nullptr;
    // a staged list is walked through its shared-memory pointer, so its
    // entries are read with shared-memory loads
    if (staged && KIND == KIND_VERLET && list_staged)
      gather_sums_staged<KIND, STEPPER == 2>(Q, B, srec, saux, L, rin, ain, q, o.cnt, slist + i, list_stride, o.r,
                                             Xi, Yi, a, nullptr, col_of, self_base);
    else if (staged)
      gather_sums_staged<KIND, STEPPER == 2>(Q, B, srec, saux, L, rin, ain, q, o.cnt, lp, list_stride, o.r, Xi, Yi,
                                             a, runs, col_of, self_base);
    else
      gather_sums<KIND, STEPPER == 2>(Q, B, rin, ain, q, o.cnt, lp, list_stride, o.r, Xi, Yi, a);
    float z[6];
    draw_noise<MODEL, STEPPER>(Q, B.ctrl->step, o.p, z);
    d2max = fmaxf(d2max, update_particle<MODEL, STEPPER>(Q, B, q, o.r, o.a, o.v, a, z, rout, aout, err,
                                                         KIND == KIND_CELLS ? B.cell_of : nullptr));
  }
}

// Staging of tile t by thread 0 (persistent launch): layout, list geometry,
// and the bulk copies of the neighbour records, aux words (AUX: SRK, which
// needs the neighbours' omega) and list rows onto the mbarrier.
template<int KIND, bool AUX>
__device__ __forceinline__ void stage_tile(const FastParams &P, const FastBuffers &B, int t, const uint4 *rin,
                                           const uint4 *ain, uint4 *srec, uint4 *saux, short *slist, uint32_t mb,
                                           TileLayout &L, int &list_staged, int &list_stride, bool reuse)
{
  L = reinterpret_cast<const TileLayout *>(B.tiles)[t];
  if (L.p_end <= L.p_begin) L.staged = 0;
  list_stride = tile_list_stride(L.p_begin, L.p_end);
  const int rows = KIND == KIND_VERLET ? B.tile_maxcnt[t] : 0;
  const uint32_t list_bytes = 2u * (uint32_t) rows * (uint32_t) list_stride;
  list_staged = L.staged && KIND == KIND_VERLET && rows > 0 && rows * list_stride <= kListCap;
  if (!L.staged) return;
  // generic-proxy reads of the buffers (previous tile) before async-proxy writes
  if (reuse) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const uint32_t tx = (AUX ? 32u : 16u) * L.total + (list_staged ? list_bytes : 0u);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(tx) : "memory");
  for (int k = 0; k < L.nseg; ++k)
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(&srec[L.base[k]])),
                 "l"(rin + L.start[k]), "r"(16u * L.len[k]), "r"(mb)
                 : "memory");
  if (AUX)
    for (int k = 0; k < L.nseg; ++k)
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_u32(&saux[L.base[k]])),
                   "l"(ain + L.start[k]), "r"(16u * L.len[k]), "r"(mb)
                   : "memory");
  if (list_staged)
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(slist)),
                 "l"(B.vl + tile_list_base(P.cap, t, L.p_begin)), "r"(list_bytes), "r"(mb)
                 : "memory");
}

// Staging of tile t by warp 0 (one launch per step): the layout read one word
// per lane, then the bulk copies issued by several lanes at once (records:
// lanes 0..5, aux words: lanes 8..13, list rows: lane 16) after lane 0 has
// armed the mbarrier with the expected bytes.  Against the same staging by
// thread 0 alone the benchmark kernel ran 0.1889 -> 0.1853 ms (same bits):
// the serial layout copy and copy issue sat on every CTA's critical path.
template<int KIND, bool AUX>
__device__ __forceinline__ void stage_tile_warp(const FastParams &P, const FastBuffers &B, int t, const uint4 *rin,
                                                const uint4 *ain, uint4 *srec, uint4 *saux, short *slist, uint32_t mb,
                                                TileLayout &L, int &list_staged, int &list_stride)
{
  constexpr int kWords = (int) (sizeof(TileLayout) / sizeof(int));
  static_assert(kWords <= 32, "one layout word per lane");
  const int lane = threadIdx.x & 31;
  const int *src = reinterpret_cast<const int *>(reinterpret_cast<const TileLayout *>(B.tiles) + t);
  if (lane < kWords) reinterpret_cast<int *>(&L)[lane] = src[lane];
  const int rows = KIND == KIND_VERLET ? B.tile_maxcnt[t] : 0;
  __syncwarp();
  const int p_begin = L.p_begin, p_end = L.p_end, total = L.total, nseg = L.nseg;
  const bool staged = L.staged && p_end > p_begin;
  const int stride = tile_list_stride(p_begin, p_end);
  const uint32_t list_bytes = 2u * (uint32_t) rows * (uint32_t) stride;
  const bool lstaged = staged && KIND == KIND_VERLET && rows > 0 && rows * stride <= kListCap;
  __syncwarp();
  if (lane == 0)
  {
    L.staged = staged ? 1 : 0;
    list_stride = stride;
    list_staged = lstaged ? 1 : 0;
    if (staged)
    {
      const uint32_t tx = (AUX ? 32u : 16u) * (uint32_t) total + (lstaged ? list_bytes : 0u);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(tx) : "memory");
    }
  }
  if (!staged) return;
  __syncwarp();
  if (lane < nseg)
  {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(&srec[L.base[lane]])),
                 "l"(rin + L.start[lane]), "r"(16u * L.len[lane]), "r"(mb)
                 : "memory");
  } else if (AUX && lane >= 8 && lane < 8 + nseg)
  {
    const int k = lane - 8;
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(&saux[L.base[k]])),
                 "l"(ain + L.start[k]), "r"(16u * L.len[k]), "r"(mb)
                 : "memory");
  } else if (lane == 16 && lstaged)
  {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(slist)),
                 "l"(B.vl + tile_list_base(P.cap, t, p_begin)), "r"(list_bytes), "r"(mb)
                 : "memory");
  }
}

__device__ __forceinline__ void init_mbarrier(uint32_t mb)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// SE or SRK step of one tile per CTA with the neighbourhood staged in shared
// memory by TMA bulk copies (cp.async.bulk, completion on an mbarrier).
// MULTI: several systems, whose parameters come from the system table (one
// system: from the kernel's parameter space, which costs no registers).
// Residency: SRK 9 CTAs per SM (56 registers, 24.7 KB of shared memory); SE
// stages no aux words (11 KB) and runs 14 CTAs per SM on cell lists (faster
// than 9, 10 or 12 despite a few spilled registers) and 10 on Verlet lists.
template<int MODEL, int STEPPER, int KIND, bool MULTI>
__global__ void __launch_bounds__(kTileThreads, STEPPER == 2 ? 9
                                                               : (KIND == KIND_VERLET ? SPSS_SE_VERLET_TILE_BLOCKS
                                                                                      : SPSS_SE_TILE_BLOCKS))
    fast_tile_kernel(FastParams P, FastBuffers B)
{
  __shared__ __align__(16) uint4 srec[kTileCap];
  __shared__ __align__(16) uint4 saux[STEPPER == 2 ? kTileCap : 1];  // aux words: SRK only (neighbour omega)
  __shared__ __align__(16) short slist[KIND == KIND_VERLET ? kListCap : 8];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ TileLayout L;
  __shared__ int list_staged, list_stride, self_base;
  __shared__ StencilRuns runs[KIND == KIND_CELLS ? kRunCells : 1];
  __shared__ unsigned char col_of[KIND == KIND_CELLS ? kTileCap : 4];
  pdl_enter();
  FastControl *ctrl = B.ctrl;
  const int par = ctrl->parity;
  const uint4 *rin = par ? B.rec1 : B.rec0;
  const uint4 *ain = par ? B.aux1 : B.aux0;
  uint4 *rout = par ? B.rec0 : B.rec1;
  uint4 *aout = par ? B.aux0 : B.aux1;
  const int t = blockIdx.x;
  const uint32_t mb = smem_u32(&mbar);
  if (threadIdx.x < 32)
  {
    if (threadIdx.x == 0) init_mbarrier(mb);
    __syncwarp();
    stage_tile_warp<KIND, STEPPER == 2>(P, B, t, rin, ain, srec, saux, slist, mb, L, list_staged, list_stride);
  }
  __syncthreads();
  const bool staged = L.staged;
  if (L.p_end <= L.p_begin) return;
  const int sys = MULTI ? B.tile_sys[t] : 0;
  const FastParams Q = MULTI ? with_system(P, B.sys[sys]) : P;
  // cell lists: the stencil run table, built while the bulk copies land
  const bool use_runs = KIND == KIND_CELLS && staged && L.ncols <= kRunCells;
  if (use_runs) build_runs(L, B.cell_off + Q.cell0, Q.nc, runs, col_of, &self_base, &ctrl->error);
  const short *glist = KIND == KIND_VERLET ? B.vl + tile_list_base(P.cap, t, L.p_begin) : nullptr;
  // the thread's first particle is loaded before the wait for the bulk
  // copies, so its global loads are in flight while the tile lands
  const int q0 = L.p_begin + threadIdx.x;
  OwnParticle o;
  if (q0 < L.p_end) o = load_own<MODEL, KIND>(B, rin, ain, q0);
  if (staged)
  {
    const uint32_t done = wait_phase(mb, 0);
    if (!__syncthreads_and(done))
    {
      // the copies did not complete in time: report, give them a second
      // bounded wait so none is in flight when the CTA exits, and stop
      if (threadIdx.x == 0) atomicOr(&ctrl->error, 2);
      wait_phase(mb, 0);
      return;
    }
  }
  float d2max = 0.0f;
  int err = 0;
  // the loop body is step_tile's, written out here: through the shared
  // function this kernel spills and runs 1 % slower
  for (int q = q0; q < L.p_end; q += blockDim.x)
  {
    if (q != q0) o = load_own<MODEL, KIND>(B, rin, ain, q);
    const unsigned p = o.p;
    const uint4 ri = o.r;
    const uint4 ai = o.a;
    const int cnt = o.cnt;
    const float2 v = o.v;
    Acc a{0.f, 0.f, 0.f, 0.f, 0};
    const uint64_t Xi = join64(ri.x, ai.x), Yi = join64(ri.y, ai.y);
    const int i = q - L.p_begin;
    const short *lp = KIND == KIND_VERLET ? (list_staged ? slist + i : glist + i) : nullptr;
    // a staged list is walked through its shared-memory pointer, so its
    // entries are read with shared-memory loads
    if (staged && KIND == KIND_VERLET && list_staged)
      gather_sums_staged<KIND, STEPPER == 2>(Q, B, srec, saux, L, rin, ain, q, cnt, slist + i, list_stride, ri, Xi,
                                             Yi, a, nullptr, col_of, self_base);
    else if (staged)
      gather_sums_staged<KIND, STEPPER == 2>(Q, B, srec, saux, L, rin, ain, q, cnt, lp, list_stride, ri, Xi, Yi, a,
                                             use_runs ? runs : nullptr, col_of, self_base);
    else
      gather_sums<KIND, STEPPER == 2>(Q, B, rin, ain, q, cnt, lp, list_stride, ri, Xi, Yi, a);
    float z[6];
    draw_noise<MODEL, STEPPER>(Q, ctrl->step, p, z);
    d2max = fmaxf(d2max, update_particle<MODEL, STEPPER>(Q, B, q, ri, ai, v, a, z, rout, aout, err,
                                                         KIND == KIND_CELLS ? B.cell_of : nullptr));
  }
  publish_max(ctrl, B.sysctl, sys, d2max, err);
}

// The same step as a persistent launch: one wave of CTAs, each taking tiles
// from a work counter until all tiles of all systems are done; the staging
// buffers and the mbarrier (one phase per staged tile) are reused.
template<int MODEL, int STEPPER, int KIND, bool MULTI>
__global__ void __launch_bounds__(kTileThreads, 8) fast_tile_persistent_kernel(FastParams P, FastBuffers B)
{
  __shared__ __align__(16) uint4 srec[kTileCap];
  __shared__ __align__(16) uint4 saux[STEPPER == 2 ? kTileCap : 1];  // aux words: SRK only (neighbour omega)
  __shared__ __align__(16) short slist[KIND == KIND_VERLET ? kListCap : 8];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ TileLayout L;
  __shared__ int list_staged, list_stride, tile_id, self_base;
  __shared__ uint32_t phase;  // mbarrier phase of the next staged tile
  __shared__ StencilRuns runs[KIND == KIND_CELLS ? kRunCells : 1];
  __shared__ unsigned char col_of[KIND == KIND_CELLS ? kTileCap : 4];
  pdl_enter();
  FastControl *ctrl = B.ctrl;
  const int par = ctrl->parity;
  const uint4 *rin = par ? B.rec1 : B.rec0;
  const uint4 *ain = par ? B.aux1 : B.aux0;
  uint4 *rout = par ? B.rec0 : B.rec1;
  uint4 *aout = par ? B.aux0 : B.aux1;
  const uint32_t mb = smem_u32(&mbar);
  if (threadIdx.x == 0)
  {
    init_mbarrier(mb);
    phase = 0;
  }
  for (bool first = true;; first = false)
  {
    if (!first) __syncthreads();  // the previous tile's shared data is no longer read
    if (threadIdx.x == 0)
    {
      const int t = atomicAdd(&ctrl->tile_next, 1);
      tile_id = t;
      if (t < P.ntiles)
        stage_tile<KIND, STEPPER == 2>(P, B, t, rin, ain, srec, saux, slist, mb, L, list_staged, list_stride,
                                       !first);
    }
    __syncthreads();
    const int t = tile_id;
    if (t >= P.ntiles) break;
    const bool staged = L.staged;
    const int sys = MULTI ? B.tile_sys[t] : 0;
    const bool use_runs = KIND == KIND_CELLS && staged && L.ncols <= kRunCells && L.p_end > L.p_begin;
    if (use_runs)
    {
      if (MULTI)
      {
        const SysParams *S = B.sys + sys;
        build_runs(L, B.cell_off + S->cell0, S->nc, runs, col_of, &self_base, &ctrl->error);
      } else
      {
        build_runs(L, B.cell_off + P.cell0, P.nc, runs, col_of, &self_base, &ctrl->error);
      }
    }
    OwnParticle o;
    if (L.p_begin + (int) threadIdx.x < L.p_end) o = load_own<MODEL, KIND>(B, rin, ain, L.p_begin + threadIdx.x);
    if (staged)
    {
      const uint32_t ph = phase;
      const uint32_t done = wait_phase(mb, ph);
      if (!__syncthreads_and(done))
      {
        if (threadIdx.x == 0) atomicOr(&ctrl->error, 2);
        wait_phase(mb, ph);
        return;
      }
      if (threadIdx.x == 0) phase = ph ^ 1u;  // read again only after the next barrier
    }
    if (L.p_end <= L.p_begin) continue;
    const short *glist = KIND == KIND_VERLET ? B.vl + tile_list_base(P.cap, t, L.p_begin) : nullptr;
    float d2max = 0.0f;
    int err = 0;
    if (!MULTI)
      step_tile<MODEL, STEPPER, KIND>(P, B, L, o, srec, saux, slist, glist, list_staged, list_stride, staged, rin,
                                      ain, rout, aout, d2max, err, use_runs ? runs : nullptr, col_of, self_base);
    else
      step_tile<MODEL, STEPPER, KIND>(with_system(P, B.sys[sys]), B, L, o, srec, saux, slist, glist, list_staged,
                                      list_stride, staged, rin, ain, rout, aout, d2max, err,
                                      use_runs ? runs : nullptr, col_of, self_base);
    publish_max(ctrl, B.sysctl, sys, d2max, err);
  }
}

// Verlet lists of one tile per CTA, from the 3x3 stencil of the rebuild grid
// (ParticleSystemFirstOrder.cpp:536-589).  The tile's neighbourhood records
// are staged in shared memory by bulk copies; each particle scans its stencil
// through the tile's run table (per stencil row at most three contiguous runs
// of staged records, in the reference's stencil order), so its list holds the
// same entries, in the same order, as the per-slot build: the staged indices
// of the neighbours with r <= r_max (widened by the guard band).  Tiles that
// are not staged, or wider than the run table, build per slot from global
// memory.  The entries go straight to global memory (L2 merges the 2-byte
// stores; assembling the rows in shared memory first measured slower).  The
// tile's longest list (rows to stage at the step) is a block maximum.
__global__ void __launch_bounds__(kTileThreads) fast_verlet_tile_build_kernel(FastParams P, FastBuffers B)
{
  __shared__ __align__(16) uint4 srec[kTileCap];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ TileLayout L;
  __shared__ int self_base, tile_max;
  __shared__ StencilRuns runs[kRunCells];
  __shared__ unsigned char col_of[kTileCap];
  FastControl *ctrl = B.ctrl;
  const int t = blockIdx.x;
  if (!rebuilds_system(B, B.tile_sys[t])) return;  // the whole CTA: its tile keeps its lists
  const uint4 *rec = ctrl->parity ? B.rec1 : B.rec0;
  const SysParams *S = B.sys + B.tile_sys[t];
  const uint32_t mb = smem_u32(&mbar);
  if (threadIdx.x == 0)
  {
    tile_max = 0;
    B.tile_maxcnt[t] = 0;  // the per-slot build below raises it
    L = reinterpret_cast<const TileLayout *>(B.tiles)[t];
    if (L.p_end <= L.p_begin || L.ncols > kRunCells) L.staged = 0;
    if (L.staged)
    {
      init_mbarrier(mb);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(16u * L.total) : "memory");
      for (int k = 0; k < L.nseg; ++k)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(&srec[L.base[k]])),
                     "l"(rec + L.start[k]), "r"(16u * L.len[k]), "r"(mb)
                     : "memory");
    }
  }
  __syncthreads();
  if (L.p_end <= L.p_begin) return;
  if (!L.staged)
  {
    for (int q = L.p_begin + threadIdx.x; q < L.p_end; q += blockDim.x) verlet_build_slot(P, B, q, t);
    return;
  }
  build_runs(L, B.cell_off + S->cell0, S->nc, runs, col_of, &self_base, &ctrl->error);
  const uint32_t done = wait_phase(mb, 0);
  if (!__syncthreads_and(done))
  {
    // the copies did not complete in time: report, wait once more so none is
    // in flight when the CTA exits, and leave the lists unbuilt
    if (threadIdx.x == 0) atomicOr(&ctrl->error, 2);
    wait_phase(mb, 0);
    return;
  }
  const float rmax2 = S->rmax2_f;
  const int stride = tile_list_stride(L.p_begin, L.p_end);
  short *const rows = B.vl + tile_list_base(P.cap, t, L.p_begin);
  int mymax = 0;
  for (int q = L.p_begin + threadIdx.x; q < L.p_end; q += blockDim.x)
  {
    const int i = q - L.p_begin;
    const int self = q + self_base;
    const uint4 ri = srec[self];
    const StencilRuns &R = runs[col_of[i]];
    int off = i;  // entry cnt of this particle at off = i + cnt * stride
    int cnt = 0;
#pragma unroll 1
    for (int r = 0; r < 3; ++r)
#pragma unroll 1
      for (int u = 0; u < 3; ++u)
      {
        const int e = R.e[r][u];
        for (int idx = R.s[r][u]; idx < e; ++idx)
        {
          const uint4 rj = srec[idx];
          const float dx = (float) (int) (rj.x - ri.x);
          const float dy = (float) (int) (rj.y - ri.y);
          if (idx != self && fmaf(dx, dx, dy * dy) <= rmax2)
          {
            if (cnt < P.cap)
            {
              rows[off] = (short) idx;
              off += stride;
            }
            ++cnt;
          }
        }
      }
    if (cnt > P.cap) atomicMax(&ctrl->overflow, cnt);
    B.vl_cnt[q] = cnt > P.cap ? -1 : cnt;
    mymax = max(mymax, min(cnt, P.cap));
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mymax = max(mymax, __shfl_xor_sync(0xffffffffu, mymax, off));
  if ((threadIdx.x & 31) == 0) atomicMax(&tile_max, mymax);
  __syncthreads();
  if (threadIdx.x == 0) B.tile_maxcnt[t] = tile_max;
}

// After a step: advance the noise counter and the buffer parity, accumulate
// each system's displacement in FP64 and set the rebuild flag
// (CalculateMaxDisplacement, ParticleSystemFirstOrder.cpp:670-696).  With
// per-system rebuilds (`selective`) a system whose trigger fires is flagged
// and restarts its own accumulator, so each system rebuilds exactly when it
// would alone; otherwise the lists of all systems are rebuilt together and
// every accumulator restarts.  One block.
// TAIL (steps run as graphs): `rebuild_exec`, the rebuild as a device graph,
// is tail-launched here when a rebuild is due, so it runs right after this
// step's graph and before the next one, and a step without a rebuild needs
// no conditional node.  A kernel that can launch a graph runs only as a node
// of a graph, so eager steps use the form without it.
template<bool TAIL>
__global__ void fast_control_kernel(FastControl *ctrl, SysControl *sysctl, const SysParams *sys, int nsys,
                                    int always_rebuild, int verlet, int selective, int cells_written,
                                    cudaGraphExec_t rebuild_exec)
{
  __shared__ int any;
  pdl_enter();
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int r = threadIdx.x; r < nsys; r += blockDim.x)
  {
    const double max2 = (double) __uint_as_float(sysctl[r].max2_bits);
    sysctl[r].max2_bits = 0u;
    if (verlet && !always_rebuild)
    {
      double acc = sysctl[r].acc + sqrt(max2);
      if (acc > sys[r].half_skin)
      {
        any = 1;
        if (selective)
        {
          sysctl[r].rebuild = 1;
          acc = 0.0;
        }
      }
      sysctl[r].acc = acc;
    }
  }
  __syncthreads();
  if (any && !selective)
    for (int r = threadIdx.x; r < nsys; r += blockDim.x) sysctl[r].acc = 0.0;
  if (threadIdx.x == 0)
  {
    ctrl->step += 1;
    ctrl->parity ^= 1;
    ctrl->tile_next = 0;
    ctrl->cells_fresh = cells_written;
    ctrl->triggered = (always_rebuild || any) ? 1 : 0;
    if (always_rebuild) ctrl->rebuild = REBUILD_ALL;
    else if (any) ctrl->rebuild = selective ? REBUILD_FLAGGED : REBUILD_ALL;
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    ctrl->acc = sysctl[0].acc;
    if (TAIL && ctrl->rebuild)
      if (cudaGraphLaunch(rebuild_exec, cudaStreamGraphTailLaunch) != cudaSuccess) atomicOr(&ctrl->error, 8);
  }
}

__global__ void fast_set_condition_kernel(const FastControl *ctrl, cudaGraphConditionalHandle handle)
{
  cudaGraphSetConditional(handle, ctrl->rebuild ? 1u : 0u);
}

__global__ void fast_noise_kernel(double *__restrict__ out, int n, int per, NoiseKey nk, const SysParams *sys,
                                  const int *sys_of)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const SysParams *S = sys + sys_of[p];
  nk.replica = (uint32_t) S->replica;
  const uint32_t local = (uint32_t) (p - S->first);
  float z[6];
  if (per > 4)
  {
    box_muller6_f32(philox_block(nk, local, 0), z);
  } else
  {
    normals4_f32(nk, local, 0, z);
  }
  for (int d = 0; d < per; ++d) out[(long) per * p + d] = (double) z[d];
}

// ApplyPeriodicBoundaryConditions: positions are kept wrapped; forget the box crossings.
__global__ void fast_pbc_kernel(int2 *img, int n)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) img[q] = make_int2(0, 0);
}

// ---------------------------------------------------------------- order parameters per system
//
// Phase order |<e^{i phi}>| and, for the second-order model, the polar order
// of the velocity directions |<v/|v|>| of every system (the observers'
// reduction, BinaryObserverFirstOrder.cpp:125-142, BinaryObserverSecondOrder.cpp:121-138),
// summed in FP64 from the records of the current state.

constexpr int kOrderChunk = 2048;  // slots per partial sum

__device__ __forceinline__ bool sample_now(const FastControl *c)
{
  return c->sample_every > 0 && (long long) c->step >= c->sample_from && (long long) c->step % c->sample_every == 0;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// partial[k] = sums over chunk k (at most kOrderChunk slots of one system);
// a small grid walks all chunks, so the gated launch that finds no sampling
// step costs a few hundred CTAs.
__global__ void fast_order_partials_kernel(FastParams P, FastBuffers B, OrderSums *__restrict__ partial,
                                           const int2 *__restrict__ items, int nitems, int gated)
{
  if (gated && !sample_now(B.ctrl)) return;
  __shared__ double sh[4][8];
  const uint4 *rec = B.ctrl->parity ? B.rec1 : B.rec0;
  for (int k = blockIdx.x; k < nitems; k += gridDim.x)
  {
    const int2 it = items[k];
    const SysParams *S = B.sys + it.x;
    const long begin = it.y;
    const long end = min((long) S->first + S->n, begin + kOrderChunk);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    for (long q = begin + threadIdx.x; q < end; q += blockDim.x)
    {
      const uint4 r = rec[q];
      a0 += (double) __uint_as_float(r.z);
      a1 += (double) __uint_as_float(r.w);
      if (P.model == 2)
      {
        const float2 v = B.vel[q];
        const double vx = v.x, vy = v.y;
        const double m = sqrt(vx * vx + vy * vy);
        if (m > 0.0)
        {
          a2 += vx / m;
          a3 += vy / m;
        }
      }
    }
    a0 = warp_sum(a0);
    a1 = warp_sum(a1);
    a2 = warp_sum(a2);
    a3 = warp_sum(a3);
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0)
    {
      sh[0][w] = a0;
      sh[1][w] = a1;
      sh[2][w] = a2;
      sh[3][w] = a3;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
      double t[4] = {0.0, 0.0, 0.0, 0.0};
      for (int u = 0; u < nw; ++u)
        for (int c = 0; c < 4; ++c) t[c] += sh[c][u];
      partial[k] = OrderSums{t[0], t[1], t[2], t[3]};
    }
    __syncthreads();
  }
}

// Per system: the order parameters (R, arg, R_v, arg_v) into out4 and, after a
// sampling step, the running sums of R, R^2, R_v, R_v^2 and the sample count.
__global__ void fast_order_finish_kernel(FastParams P, FastBuffers B, const OrderSums *__restrict__ partial,
                                         const int *__restrict__ first_item, double *__restrict__ out4,
                                         double *__restrict__ stats, int gated)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= P.nsys) return;
  if (gated && !sample_now(B.ctrl)) return;
  double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
  for (int c = first_item[r]; c < first_item[r + 1]; ++c)
  {
    const OrderSums v = partial[c];
    t0 += v.c;
    t1 += v.s;
    t2 += v.vx;
    t3 += v.vy;
  }
  const double n = (double) B.sys[r].n;
  const double re = t0 / n, im = t1 / n;
  double o[4];
  o[0] = sqrt(re * re + im * im);
  o[1] = atan2(im, re);
  if (P.model == 2)
  {
    const double vre = t2 / n, vim = t3 / n;
    o[2] = sqrt(vre * vre + vim * vim);
    o[3] = atan2(vim, vre);
  } else
  {
    o[2] = o[0];
    o[3] = o[1];
  }
  for (int k = 0; k < 4; ++k) out4[4 * r + k] = o[k];
  if (gated)
  {
    double *st = stats + 5 * r;
    st[0] += o[0];
    st[1] += o[0] * o[0];
    st[2] += o[2];
    st[3] += o[2] * o[2];
    st[4] += 1.0;
  }
}

// ---------------------------------------------------------------- global polar order field
//
// EvaluateInteractionsWithGlobalPolarOrderField (ParticleSystemFirstOrderPtr.cpp:155-223):
// every particle couples to Z = <e^{i phi}> (and, for the complementary force
// of the SRK stepper, to W = <omega e^{i phi}>), both summed in FP64 over the
// stage state; no lists.

constexpr int kFieldBlocks = 304;

__global__ void fast_field_partials_kernel(FastParams P, FastBuffers B)
{
  __shared__ double sh[4][8];
  const int par = B.ctrl->parity;
  const uint4 *rec = par ? B.rec1 : B.rec0;
  const uint4 *aux = par ? B.aux1 : B.aux0;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < P.n; q += gridDim.x * blockDim.x)
  {
    const double c = (double) __uint_as_float(rec[q].z), sn = (double) __uint_as_float(rec[q].w);
    const double w = (double) __uint_as_float(aux[q].w);
    a0 += c;
    a1 += sn;
    a2 += w * c;
    a3 += w * sn;
  }
  a0 = warp_sum(a0);
  a1 = warp_sum(a1);
  a2 = warp_sum(a2);
  a3 = warp_sum(a3);
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0)
  {
    sh[0][wid] = a0;
    sh[1][wid] = a1;
    sh[2][wid] = a2;
    sh[3][wid] = a3;
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < nw; ++k)
      for (int c = 0; c < 4; ++c) t[c] += sh[c][k];
    for (int c = 0; c < 4; ++c) B.field_partial[4 * blockIdx.x + c] = t[c];
  }
}

// field = {Re Z, Im Z, |Z|, Re W, Im W, |W|, cos arg W, sin arg W}
__global__ void fast_field_finish_kernel(FastParams P, FastBuffers B)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = 0; b < kFieldBlocks; ++b)
    for (int c = 0; c < 4; ++c) t[c] += B.field_partial[4 * b + c];
  const double zr = t[0] / P.n, zi = t[1] / P.n, wr = t[2] / P.n, wi = t[3] / P.n;
  const double aw = atan2(wi, wr);  // arg 0 = 0, as std::arg
  B.field[0] = zr;
  B.field[1] = zi;
  B.field[2] = sqrt(zr * zr + zi * zi);
  B.field[3] = wr;
  B.field[4] = wi;
  B.field[5] = sqrt(wr * wr + wi * wi);
  B.field[6] = cos(aw);
  B.field[7] = sin(aw);
}

// One SE or SRK step of the first-order model in the global field:
// k[3] = -xi omega + nu_i + sigma |Z| (sin(arg Z - phi) cos a - cos(arg Z - phi) sin a)
// and the complementary force as the reference computes it, whose last term
// takes sin(arg W - phi) (ParticleSystemFirstOrderPtr.cpp:213-219).
template<int STEPPER>
__global__ void __launch_bounds__(kTB, 4) fast_global_step_kernel(FastParams P, FastBuffers B)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  FastControl *ctrl = B.ctrl;
  const int par = ctrl->parity;
  const uint4 *rin = par ? B.rec1 : B.rec0;
  const uint4 *ain = par ? B.aux1 : B.aux0;
  uint4 *rout = par ? B.rec0 : B.rec1;
  uint4 *aout = par ? B.aux0 : B.aux1;
  float d2max = 0.0f;
  int err = 0;
  if (q < P.n)
  {
    const unsigned p = B.pid[q];
    const uint4 ri = rin[q];
    const uint4 ai = ain[q];
    float z[6];
    draw_noise<1, STEPPER>(P, ctrl->step, p, z);
    const float zr = (float) B.field[0], zi = (float) B.field[1], az = (float) B.field[2];
    const float wr = (float) B.field[3], wim = (float) B.field[4], aw = (float) B.field[5];
    const float cw = (float) B.field[6], sw = (float) B.field[7];
    const float cphi = __uint_as_float(ri.z), sphi = __uint_as_float(ri.w), wi = __uint_as_float(ai.w);
    const float SZ = fmaf(zi, cphi, -__fmul_rn(zr, sphi));  // |Z| sin(arg Z - phi)
    const float KZ = fmaf(zr, cphi, __fmul_rn(zi, sphi));   // |Z| cos(arg Z - phi)
    const float f_w = fmaf(-P.xi_phi, wi, __fadd_rn(B.nu[q], __fmul_rn(P.sigma, fmaf(P.ca, SZ, -__fmul_rn(P.sa, KZ)))));
    float C = 0.0f;
    if (STEPPER == 2)
    {
      const float KW = fmaf(wr, cphi, __fmul_rn(wim, sphi));   // |W| cos(arg W - phi)
      const float sWp = fmaf(sw, cphi, -__fmul_rn(cw, sphi));  // sin(arg W - phi)
      const float first = fmaf(P.ca, KW, __fmul_rn(P.sa, __fmul_rn(aw, sWp)));
      const float second = __fmul_rn(wi, fmaf(P.ca, KZ, __fmul_rn(P.sa, __fmul_rn(az, sWp))));
      C = __fmul_rn(P.sigma, __fsub_rn(first, second));
    }
    d2max = advance_particle<1, STEPPER>(P, B, q, ri, ai, make_float2(0.f, 0.f), f_w, C, z, rout, aout, err);
  }
  publish_max(ctrl, B.sysctl, 0, d2max, err);
}

__global__ void fast_set_frequencies_kernel(const double *__restrict__ freqs, int n, float *__restrict__ nu)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) nu[i] = (float) freqs[i];
}

// ---------------------------------------------------------------- host side

static int blocks_for(long n, int tb)
{
  return (int) ((n + tb - 1) / tb);
}

static bool has_cells(int kind)
{
  return kind == KIND_CELLS || kind == KIND_VERLET;
}

static FastBuffers buffers(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  FastBuffers B;
  B.rec0 = f->rec[0].ptr;
  B.rec1 = f->rec[1].ptr;
  B.aux0 = f->aux[0].ptr;
  B.aux1 = f->aux[1].ptr;
  B.vel = f->vel.ptr;
  B.vel_tmp = f->vel_tmp.ptr;
  B.pid = f->pid.ptr;
  B.pid_tmp = f->pid_tmp.ptr;
  B.inv = f->inv.ptr;
  B.img = f->img.ptr;
  B.turns = f->turns.ptr;
  B.cell_of = f->cell_of.ptr;
  B.cell_sorted = f->cell_sorted.ptr;
  B.cell_off = f->binner.offsets.ptr;
  B.order = f->binner.members.ptr;
  B.vl = f->vl.ptr;
  B.vl_cnt = f->vl_cnt.ptr;
  B.tile_maxcnt = f->tile_maxcnt.ptr;
  B.tiles = f->tiles.ptr;
  B.sys = f->sys.ptr;
  B.sys_of = f->sys_of.ptr;
  B.tile_sys = f->tile_sys.ptr;
  B.sysctl = f->sysctl.ptr;
  B.nu = f->nu.ptr;
  B.field = f->field.ptr;
  B.field_partial = f->field_partial.ptr;
  B.ctrl = f->ctrl;
  return B;
}

// Table entry of one system: its parameters in the FP32 / fixed-point units
// of the kernels.
static SysParams system_params(const spss_params &p, int index, int first, int nc, int cell0, int tile0,
                               int ntiles, double r_min, double r_max)
{
  SysParams S;
  std::memset(&S, 0, sizeof(S));
  S.n = p.n;
  S.first = first;
  S.nc = nc;
  S.cell0 = cell0;
  S.tile0 = tile0;
  S.ntiles = ntiles;
  S.index = index;
  S.replica = (int) p.replica;
  S.v0 = (float) p.v0;
  S.xi = (float) p.xi;
  S.xi_r = (float) p.xi_r;
  // first order: the torque friction is xi; second order: xi_phi
  S.xi_phi = (float) (p.model == 1 ? p.xi : p.xi_phi);
  S.sigma = (float) p.sigma;
  S.ca = (float) std::cos(p.alpha);
  S.sa = (float) std::sin(p.alpha);
  const double rho2 = p.rho * p.rho;
  S.rho2_d = rho2;
  // FP32 pair distances are squared differences of the 32-bit position words,
  // i.e. in units of 2^-64 of the box area
  const double area = 18446744073709551616.0;
  S.rho2_f = (float) (rho2 * area);
  // |d2_f - d2| <= 2 (|dx| + |dy|) 2^-32 + 2^-32 + 4 d2 2^-24 near r = rho; doubled
  S.band_f = (float) (area * 2.0 * (4.0 * p.rho * 2.3283064365386963e-10 + 2.3283064365386963e-10 + 4.0 * rho2 * 5.9604644775390625e-8));
  const double rmax2 = r_max * r_max;
  S.rmax2_f = (float) (area * (rmax2 + 2.0 * (4.0 * r_max * 2.3283064365386963e-10 + 4.0 * rmax2 * 5.9604644775390625e-8)));
  S.half_skin = 0.5 * (r_max - r_min);
  S.b_r = (float) std::sqrt(2.0 * p.D_r);
  S.b_phi = (float) std::sqrt(2.0 * p.D_phi);
  return S;
}

static FastParams params(spss_ctx *ctx, double dt)
{
  const spss_params &p = ctx->p;
  FastPath *f = ctx->fast;
  const SysParams &S = f->h_sys[0];
  FastParams P;
  std::memset(&P, 0, sizeof(P));
  P.n = p.n;
  P.cap = f->cap;
  P.model = p.model;
  P.kind = f->kind;
  P.always_rebuild = f->kind == KIND_CELLS ? 1 : 0;
  P.selective = f->nsys > 1 && f->kind == KIND_VERLET ? 1 : 0;
  P.tile_cells = f->tile_cells;
  P.persistent = f->persistent;
  P.nsys = f->nsys;
  P.ntiles = f->ntiles;
  // system 0 (kernels that serve several systems read theirs from the table)
  P.nc = S.nc;
  P.first = S.first;
  P.sub_n = S.n;
  P.cell0 = S.cell0;
  P.v0 = S.v0;
  P.xi = S.xi;
  P.xi_r = S.xi_r;
  P.xi_phi = S.xi_phi;
  P.sigma = S.sigma;
  P.ca = S.ca;
  P.sa = S.sa;
  P.rho2_f = S.rho2_f;
  P.band_f = S.band_f;
  P.rmax2_f = S.rmax2_f;
  P.rho2_d = S.rho2_d;
  P.half_skin = S.half_skin;
  P.b_r = S.b_r;
  P.b_phi = S.b_phi;
  P.dt = (float) dt;
  P.sqdt = (float) std::sqrt(dt);
  P.half_dt2 = (float) (0.5 * dt * dt);
  P.half_dt15 = (float) (0.5 * std::pow(dt, 1.5));
  P.inv_sqrt3 = (float) (1.0 / std::sqrt(3.0));
  P.seed = p.seed;
  philox_round_keys(p.seed, P.kx, P.ky);
  P.replica = (uint32_t) S.replica;
  return P;
}

// Tile tables for a tile width (cells per tile); every system's tiles follow
// the previous system's.
static int set_tiling(spss_ctx *ctx, int tile_cells)
{
  FastPath *f = ctx->fast;
  if (f->kind == KIND_ALL_PAIRS || f->kind == KIND_GLOBAL) return SPSS_OK;
  f->tile_cells = tile_cells;
  int ntiles = 0;
  std::vector<int> tile_sys;
  for (int r = 0; r < f->nsys; ++r)
  {
    SysParams &S = f->h_sys[r];
    S.tile0 = ntiles;
    S.ntiles = S.nc * tiles_per_row(S.nc, tile_cells);
    ntiles += S.ntiles;
    tile_sys.insert(tile_sys.end(), (size_t) S.ntiles, r);
  }
  f->ntiles = ntiles;
  SPSS_TRY(f->tiles.reserve(sizeof(TileLayout) * (size_t) ntiles));
  SPSS_TRY(f->tile_sys.reserve((size_t) ntiles));
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->tile_sys.ptr, tile_sys.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice,
                                ctx->stream));
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->sys.ptr, f->h_sys.data(), sizeof(SysParams) * f->nsys, cudaMemcpyHostToDevice,
                                ctx->stream));
  if (f->kind == KIND_VERLET)
  {
    SPSS_TRY(f->vl.reserve((size_t) f->cap * ((size_t) ctx->p.n + 16 * (size_t) ntiles + 16)));
    SPSS_TRY(f->tile_maxcnt.reserve((size_t) ntiles));
  }
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  // lists and layouts follow the tiles: rebuild before the next step
  f->h_ctrl->rebuild = 1;
  ctx->should_update_lists = 1;
  SPSS_CUDA_TRY(cudaMemcpyAsync(&f->ctrl->rebuild, &f->h_ctrl->rebuild, sizeof(int), cudaMemcpyHostToDevice,
                                ctx->stream));
  for (auto &g : f->graphs) g.second.release();
  f->graphs.clear();
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int fast_create(spss_ctx *ctx)
{
  FastPath *f = new FastPath();
  ctx->fast = f;
  const spss_params &p = ctx->p;
  const int n = p.n;
  std::vector<spss_params> systems = ctx->systems;
  if (systems.empty()) systems.push_back(p);
  f->nsys = (int) systems.size();
  int kind = -1;
  double lam_max = 0.0;
  int first = 0, cell0 = 0;
  for (int r = 0; r < f->nsys; ++r)
  {
    const spss_params &q = systems[r];
    double r_min, r_max;
    int nc, nc_verlet;
    derive_lists(q, r_min, r_max, nc, nc_verlet);
    int k, grid;
    switch (variant_for_params(q, q.variant))
    {
      case SPSS_VARIANT_ALL_PAIRS:
        k = KIND_ALL_PAIRS;
        grid = 1;
        break;
      case SPSS_VARIANT_LINKED_LIST:
        k = KIND_CELLS;
        grid = nc;
        break;
      case SPSS_VARIANT_VERLET:
        // O(N^2) list build = every pair within r_max: cells no smaller than r_max.  With fewer
        // than three such cells per side (r_max > 1/3: the reference's first-order dispatch for
        // 0.25 < rho <= 0.5, ParticleSystemFirstOrder.cpp:96-111) a list holds a third of the
        // system or more and the stencil would visit cells twice: every pair is evaluated each
        // step instead, the same neighbours within rho, with the list trigger kept.
        grid = std::max(1, (int) (1.0 / r_max));
        k = grid < 3 ? KIND_ALL_PAIRS : KIND_VERLET;
        if (grid < 3)
        {
          grid = 1;
          f->trigger_only = true;
        }
        break;
      case SPSS_VARIANT_LINKED_LIST_VERLET:
        k = KIND_VERLET;
        grid = nc_verlet;
        break;
      case SPSS_VARIANT_GLOBAL_FIELD:
        // the reference's global field belongs to the first-order model; one system
        if (q.model != 1 || systems.size() != 1) return SPSS_ERR_NOT_SUPPORTED;
        k = KIND_GLOBAL;
        grid = 1;
        break;
      default:
        return SPSS_ERR_NOT_SUPPORTED;
    }
    if (kind >= 0 && k != kind) return SPSS_ERR_NOT_SUPPORTED;  // one list kind per context
    kind = k;
    if ((long) cell0 + (long) grid * grid > 0x7fffffffL) return SPSS_ERR_SIZE;
    f->h_sys.push_back(system_params(q, r, first, grid, cell0, 0, 0, r_min, r_max));
    first += q.n;
    cell0 += grid * grid;
    lam_max = std::max(lam_max, M_PI * r_max * r_max * q.n);
  }
  if (first != n) return SPSS_ERR_INVALID_ARGUMENT;
  f->kind = kind;
  f->total_cells = cell0;
  if (kind == KIND_GLOBAL)
  {
    SPSS_TRY(f->nu.reserve((size_t) n));
    SPSS_TRY(f->field.reserve(8));
    SPSS_TRY(f->field_partial.reserve(4 * kFieldBlocks));
    SPSS_CUDA_TRY(cudaMemsetAsync(f->nu.ptr, 0, sizeof(float) * n, ctx->stream));
  }
  f->nc_build = f->h_sys[0].nc;
  if (f->kind == KIND_VERLET || f->trigger_only) ctx->uses_verlet_list = 1;
  for (int b = 0; b < 2; ++b)
  {
    SPSS_TRY(f->rec[b].reserve(n));
    SPSS_TRY(f->aux[b].reserve(n));
  }
  SPSS_TRY(f->vel.reserve(n));
  SPSS_TRY(f->vel_tmp.reserve(n));
  SPSS_TRY(f->pid.reserve(n));
  SPSS_TRY(f->pid_tmp.reserve(n));
  SPSS_TRY(f->inv.reserve(n));
  SPSS_TRY(f->img.reserve(n));
  SPSS_TRY(f->turns.reserve(n));
  SPSS_TRY(f->cell_of.reserve(n));
  SPSS_TRY(f->cell_sorted.reserve(n));
  SPSS_TRY(f->vl_cnt.reserve(n));
  SPSS_TRY(f->sys.reserve((size_t) f->nsys));
  SPSS_TRY(f->sysctl.reserve((size_t) f->nsys));
  SPSS_TRY(f->sys_of.reserve((size_t) n));
  {
    std::vector<int2> items;
    std::vector<int> first_item;
    for (const SysParams &S : f->h_sys)
    {
      first_item.push_back((int) items.size());
      for (long b = 0; b < S.n; b += kOrderChunk) items.push_back(make_int2(S.index, (int) (S.first + b)));
    }
    first_item.push_back((int) items.size());
    f->order_chunks = (int) items.size();
    f->order_grid = std::min(f->order_chunks, 4 * 152);
    SPSS_TRY(f->order_partial.reserve((size_t) f->order_chunks));
    SPSS_TRY(f->order_items.reserve(items.size()));
    SPSS_TRY(f->order_first.reserve(first_item.size()));
    SPSS_CUDA_TRY(cudaMemcpyAsync(f->order_items.ptr, items.data(), sizeof(int2) * items.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
    SPSS_CUDA_TRY(cudaMemcpyAsync(f->order_first.ptr, first_item.data(), sizeof(int) * first_item.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
    SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    SPSS_TRY(f->order_out.reserve((size_t) f->nsys * 4));
    SPSS_TRY(f->stats.reserve((size_t) f->nsys * 5));
    SPSS_CUDA_TRY(cudaMemsetAsync(f->stats.ptr, 0, sizeof(double) * 5 * f->nsys, ctx->stream));
  }
  if (f->kind == KIND_VERLET)
  {
    // mean list length: pi r_max^2 n (unit box); room for six standard deviations
    f->cap = std::max(16, ((int) std::ceil(lam_max + 6.0 * std::sqrt(lam_max) + 8.0) + 3) & ~3);
  }
  {
    std::vector<int> sys_of((size_t) n);
    for (int r = 0; r < f->nsys; ++r)
      std::fill(sys_of.begin() + f->h_sys[r].first, sys_of.begin() + f->h_sys[r].first + f->h_sys[r].n, r);
    SPSS_CUDA_TRY(cudaMemcpyAsync(f->sys_of.ptr, sys_of.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  SPSS_CUDA_TRY(cudaMemsetAsync(f->sysctl.ptr, 0, sizeof(SysControl) * f->nsys, ctx->stream));
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->sys.ptr, f->h_sys.data(), sizeof(SysParams) * f->nsys, cudaMemcpyHostToDevice,
                                ctx->stream));
  SPSS_CUDA_TRY(cudaMalloc((void **) &f->ctrl, sizeof(FastControl)));
  SPSS_CUDA_TRY(cudaMallocHost((void **) &f->h_ctrl, sizeof(FastControl)));
  std::memset(f->h_ctrl, 0, sizeof(FastControl));
  f->h_ctrl->rebuild = 1;
  f->h_ctrl->uses_verlet = f->kind == KIND_VERLET;
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->ctrl, f->h_ctrl, sizeof(FastControl), cudaMemcpyHostToDevice, ctx->stream));
  SPSS_CUDA_TRY(cudaMemsetAsync(f->vel.ptr, 0, sizeof(float2) * n, ctx->stream));
  SPSS_TRY(set_tiling(ctx, kTileCellsDefault));
  // resident CTAs of the persistent tile kernel: one wave
  {
    int dev = 0, sms = 0, per_sm = 0;
    SPSS_CUDA_TRY(cudaGetDevice(&dev));
    SPSS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SPSS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fast_tile_persistent_kernel<2, 2, KIND_VERLET, true>,
                                                                kTileThreads, 0));
    f->persistent_grid = std::max(1, sms * std::max(1, per_sm));
  }
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

void fast_destroy(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  if (!f) return;
  for (auto &g : f->graphs) g.second.release();
  for (int b = 0; b < 2; ++b)
  {
    f->rec[b].release();
    f->aux[b].release();
  }
  f->vel.release();
  f->vel_tmp.release();
  f->pid.release();
  f->pid_tmp.release();
  f->inv.release();
  f->img.release();
  f->turns.release();
  f->cell_of.release();
  f->cell_sorted.release();
  f->vl.release();
  f->vl_cnt.release();
  f->tile_maxcnt.release();
  f->tiles.release();
  f->sys.release();
  f->sys_of.release();
  f->tile_sys.release();
  f->sysctl.release();
  f->nu.release();
  f->field.release();
  f->field_partial.release();
  f->order_partial.release();
  f->order_items.release();
  f->order_first.release();
  f->order_out.release();
  f->stats.release();
  f->snap.release();
  f->binner.release();
  if (f->ctrl) cudaFree(f->ctrl);
  if (f->h_ctrl) cudaFreeHost(f->h_ctrl);
  delete f;
  ctx->fast = nullptr;
}

// Cell binning, slot re-sort and (Verlet) list build, as one stream sequence.
static int launch_rebuild(spss_ctx *ctx, const FastParams &P)
{
  FastPath *f = ctx->fast;
  const FastBuffers B = buffers(ctx);
  const int n = P.n;
  if (has_cells(f->kind))
  {
    fast_cells_kernel<<<blocks_for(n, kTB), kTB, 0, ctx->stream>>>(P, B);
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_cells_kernel"));
    SPSS_TRY(f->binner.run(f->cell_of.ptr, n, f->total_cells, ctx->stream, ctx->launches, f->chain));
    const FastBuffers B2 = buffers(ctx);  // binner buffers exist now
    SPSS_CUDA_TRY(launch_chained(f->chain, fast_permute_kernel, blocks_for(n, kTB), kTB, 0, ctx->stream, P, B2));
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_permute_kernel"));
    SPSS_CUDA_TRY(launch_chained(f->chain, fast_copyback_kernel, blocks_for(n, kTB), kTB, 0, ctx->stream, P, B2));
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_copyback_kernel"));
  }
  SPSS_CUDA_TRY(launch_chained(f->chain, fast_after_permute_kernel, 1, 1, 0, ctx->stream, f->ctrl,
                               (int) has_cells(f->kind)));
  ++ctx->launches;
  SPSS_TRY(check_launch("fast_after_permute_kernel"));
  if (has_cells(f->kind))
  {
    SPSS_CUDA_TRY(launch_chained(f->chain, fast_tile_layout_kernel, blocks_for(f->ntiles, 128), 128, 0, ctx->stream,
                                 P, buffers(ctx)));
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_tile_layout_kernel"));
  }
  if (f->kind == KIND_VERLET)
  {
    fast_verlet_tile_build_kernel<<<f->ntiles, kTileThreads, 0, ctx->stream>>>(P, buffers(ctx));
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_verlet_tile_build_kernel"));
  }
  SPSS_CUDA_TRY(launch_chained(f->chain, fast_after_rebuild_kernel, 1, 256, 0, ctx->stream, f->ctrl, f->sysctl.ptr,
                               f->nsys));
  ++ctx->launches;
  return check_launch("fast_after_rebuild_kernel");
}

template<int MODEL, int STEPPER, int KIND>
static void launch_tiles(spss_ctx *ctx, const FastParams &P, const FastBuffers &B, int grid)
{
  const bool c = ctx->fast->chain;
  if (P.persistent)
  {
    if (P.nsys > 1)
      launch_chained(c, fast_tile_persistent_kernel<MODEL, STEPPER, KIND, true>, grid, kTileThreads, 0, ctx->stream, P, B);
    else
      launch_chained(c, fast_tile_persistent_kernel<MODEL, STEPPER, KIND, false>, grid, kTileThreads, 0, ctx->stream, P,
                     B);
  } else
  {
    if (P.nsys > 1)
      launch_chained(c, fast_tile_kernel<MODEL, STEPPER, KIND, true>, grid, kTileThreads, 0, ctx->stream, P, B);
    else
      launch_chained(c, fast_tile_kernel<MODEL, STEPPER, KIND, false>, grid, kTileThreads, 0, ctx->stream, P, B);
  }
}

template<int MODEL, int STEPPER>
static void launch_step_kind(spss_ctx *ctx, const FastParams &P, const FastBuffers &B)
{
  const int grid = blocks_for(P.n, kTB);
  const int tiles = P.persistent ? std::min(P.ntiles, ctx->fast->persistent_grid) : P.ntiles;
  if (ctx->fast->kind == KIND_GLOBAL)
  {
    if (MODEL == 1)
    {
      fast_field_partials_kernel<<<kFieldBlocks, 256, 0, ctx->stream>>>(P, B);
      fast_field_finish_kernel<<<1, 32, 0, ctx->stream>>>(P, B);
      fast_global_step_kernel<STEPPER><<<grid, kTB, 0, ctx->stream>>>(P, B);
      ctx->launches += 2;
    }
  } else if (ctx->fast->kind == KIND_ALL_PAIRS)
  {
    if (P.nsys > 1) fast_step_kernel<MODEL, STEPPER, KIND_ALL_PAIRS, true><<<grid, kTB, 0, ctx->stream>>>(P, B);
    else fast_step_kernel<MODEL, STEPPER, KIND_ALL_PAIRS, false><<<grid, kTB, 0, ctx->stream>>>(P, B);
  } else if (ctx->fast->kind == KIND_CELLS)
  {
    launch_tiles<MODEL, STEPPER, KIND_CELLS>(ctx, P, B, tiles);
  } else
  {
    launch_tiles<MODEL, STEPPER, KIND_VERLET>(ctx, P, B, tiles);
  }
}

static int launch_step(spss_ctx *ctx, int stepper, const FastParams &P, cudaGraphExec_t rebuild_exec = nullptr)
{
  const FastBuffers B = buffers(ctx);
  if (ctx->timing) SPSS_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
  if (ctx->p.model == 1)
  {
    if (stepper == SPSS_STEPPER_STOCHASTIC_EULER) launch_step_kind<1, 1>(ctx, P, B);
    else launch_step_kind<1, 2>(ctx, P, B);
  } else
  {
    if (stepper == SPSS_STEPPER_STOCHASTIC_EULER) launch_step_kind<2, 1>(ctx, P, B);
    else launch_step_kind<2, 2>(ctx, P, B);
  }
  ++ctx->launches;
  SPSS_TRY(check_launch("fast_step_kernel"));
  if (ctx->timing) SPSS_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
  FastPath *f = ctx->fast;
  if (rebuild_exec)
    fast_control_kernel<true><<<1, 256, 0, ctx->stream>>>(f->ctrl, f->sysctl.ptr, f->sys.ptr, f->nsys,
                                                          P.always_rebuild, f->kind == KIND_VERLET || f->trigger_only,
                                                          P.selective, f->kind == KIND_CELLS ? 1 : 0, rebuild_exec);
  else
    launch_chained(f->chain, fast_control_kernel<false>, 1, 256, 0, ctx->stream, f->ctrl, f->sysctl.ptr,
                   (const SysParams *) f->sys.ptr, f->nsys, (int) P.always_rebuild,
                   (int) (f->kind == KIND_VERLET || f->trigger_only), (int) P.selective,
                   f->kind == KIND_CELLS ? 1 : 0, (cudaGraphExec_t) nullptr);
  ++ctx->launches;
  return check_launch("fast_control_kernel");
}

// Order parameters of every system; `gated`: only after a sampling step, and
// then also added to the running averages.
static int launch_sampling(spss_ctx *ctx, const FastParams &P, int gated)
{
  FastPath *f = ctx->fast;
  const FastBuffers B = buffers(ctx);
  fast_order_partials_kernel<<<f->order_grid, 256, 0, ctx->stream>>>(P, B, f->order_partial.ptr,
                                                                       f->order_items.ptr, f->order_chunks, gated);
  ++ctx->launches;
  SPSS_TRY(check_launch("fast_order_partials_kernel"));
  fast_order_finish_kernel<<<blocks_for(f->nsys, 128), 128, 0, ctx->stream>>>(
      P, B, f->order_partial.ptr, f->order_first.ptr, f->order_out.ptr, f->stats.ptr, gated);
  ++ctx->launches;
  return check_launch("fast_order_finish_kernel");
}

// The reference's should_update_lists after a step: set by the trigger until
// the next evaluation rebuilds.  A graph step performs its rebuild at once
// (tail launch), so the flag reads from the trigger of the last step as well.
static int reported_list_flag(const FastControl *c)
{
  return (c->rebuild || c->triggered) ? 1 : 0;
}

static int sync_control(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->h_ctrl, f->ctrl, sizeof(FastControl), cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ctx->step_counter = f->h_ctrl->step;
  ctx->accumulated_displacement = f->h_ctrl->acc;
  ctx->should_update_lists = reported_list_flag(f->h_ctrl);
  if (f->h_ctrl->error & ~1) return SPSS_ERR_CUDA;  // a bounded wait ran out, or a device launch failed
  if (f->h_ctrl->error) return SPSS_ERR_NONFINITE;
  return SPSS_OK;
}

// The host-side step counter and list flag (spss_set_step_counter,
// spss_set_should_update_lists) win over the device copy.
static int push_host_control(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  if (f->h_ctrl->step == ctx->step_counter && reported_list_flag(f->h_ctrl) == ctx->should_update_lists)
    return SPSS_OK;
  if (reported_list_flag(f->h_ctrl) != ctx->should_update_lists)
  {
    f->h_ctrl->rebuild = ctx->should_update_lists ? REBUILD_ALL : REBUILD_NONE;
    f->h_ctrl->triggered = 0;
  }
  f->h_ctrl->step = ctx->step_counter;
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->ctrl, f->h_ctrl, sizeof(FastControl), cudaMemcpyHostToDevice, ctx->stream));
  return SPSS_OK;
}

int fast_set_state(spss_ctx *ctx, const double *d_aos)
{
  FastPath *f = ctx->fast;
  fast_upload_kernel<<<blocks_for(ctx->p.n, kTB), kTB, sizeof(double) * kTB * ctx->s, ctx->stream>>>(
      d_aos, ctx->p.n, ctx->s, ctx->p.model, f->perm_valid ? 1 : 0, buffers(ctx));
  ++ctx->launches;
  SPSS_TRY(check_launch("fast_upload_kernel"));
  // new positions: the next cell-list rebuild computes the cell ids
  f->h_ctrl->cells_fresh = 0;
  SPSS_CUDA_TRY(cudaMemsetAsync(&f->ctrl->cells_fresh, 0, sizeof(int), ctx->stream));
  // the last step's trigger fired and a graph step already rebuilt the lists
  // from the positions before this upload: the reference rebuilds from the
  // state it is given next, so rebuild again before the next step
  if (f->h_ctrl->triggered && !f->h_ctrl->rebuild)
  {
    f->h_ctrl->rebuild = REBUILD_ALL;
    SPSS_CUDA_TRY(cudaMemcpyAsync(&f->ctrl->rebuild, &f->h_ctrl->rebuild, sizeof(int), cudaMemcpyHostToDevice,
                                  ctx->stream));
  }
  f->perm_valid = true;
  f->have_state = true;
  return SPSS_OK;
}

int fast_get_state(spss_ctx *ctx, double *d_aos)
{
  fast_download_kernel<<<blocks_for(ctx->p.n, kTB), kTB, sizeof(double) * kTB * ctx->s, ctx->stream>>>(
      d_aos, ctx->p.n, ctx->s, ctx->p.model, buffers(ctx));
  ++ctx->launches;
  return check_launch("fast_download_kernel");
}

int fast_step(spss_ctx *ctx, int stepper, double t, double dt)
{
  (void) t;
  FastPath *f = ctx->fast;
  if (!f->have_state) return SPSS_ERR_INVALID_ARGUMENT;
  if (stepper == SPSS_STEPPER_RK4) return SPSS_ERR_NOT_SUPPORTED;
  const FastParams P = params(ctx, dt);
  SPSS_TRY(push_host_control(ctx));
  if (f->h_ctrl->rebuild) SPSS_TRY(launch_rebuild(ctx, P));
  SPSS_TRY(launch_step(ctx, stepper, P));
  const int rc = sync_control(ctx);
  if (ctx->timing)
  {
    float ms = 0.0f;
    SPSS_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->timing_ms += ms;
    ctx->timing_count += 1;
  }
  return rc;
}

static int build_graph_on(spss_ctx *ctx, int stepper, const FastParams &P, int sampling, GraphEntry &g,
                          unsigned long long launches0);

// One step as a graph (+ the gated order-parameter sample): on a rebuild
// trigger, step + control, the control kernel tail-launching the rebuild graph
// when it is due (or the conditional form, whose rebuild sits under a
// conditional node ahead of the step); with cell lists, rebuild + step +
// control; otherwise step + control.
static int build_graph(spss_ctx *ctx, int stepper, double dt, int sampling, GraphEntry &g)
{
  const FastParams P = params(ctx, dt);
  const unsigned long long launches0 = ctx->launches;
  const int timing = ctx->timing;
  cudaStream_t work = ctx->stream;
  ctx->timing = 0;
  ctx->stream = ctx->own_stream;  // capture needs a non-legacy stream
  int rc_all = build_graph_on(ctx, stepper, P, sampling, g, launches0);
  ctx->stream = work;
  ctx->timing = timing;
  return rc_all;
}

// The conditional form: set-condition kernel, IF rebuild, step and control.
static int build_graph_conditional(spss_ctx *ctx, int stepper, const FastParams &P, int sampling, GraphEntry &g,
                                   unsigned long long launches0)
{
  FastPath *f = ctx->fast;
  cudaGraph_t graph;
  SPSS_CUDA_TRY(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle handle;
  SPSS_CUDA_TRY(cudaGraphConditionalHandleCreate(&handle, graph, 0, cudaGraphCondAssignDefault));
  // node 1: copy the rebuild flag into the condition
  SPSS_CUDA_TRY(cudaStreamBeginCaptureToGraph(ctx->stream, graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  fast_set_condition_kernel<<<1, 1, 0, ctx->stream>>>(f->ctrl, handle);
  ++ctx->launches;
  SPSS_CUDA_TRY(cudaStreamEndCapture(ctx->stream, &graph));
  size_t nnodes = 0;
  SPSS_CUDA_TRY(cudaGraphGetNodes(graph, nullptr, &nnodes));
  std::vector<cudaGraphNode_t> nodes(nnodes);
  SPSS_CUDA_TRY(cudaGraphGetNodes(graph, nodes.data(), &nnodes));
  cudaGraphNode_t set_node = nodes.back();
  // node 2: IF rebuild
  // the struct holds a union with deleted constructors: zeroed raw storage
  alignas(cudaGraphNodeParams) unsigned char cp_storage[sizeof(cudaGraphNodeParams)] = {};
  cudaGraphNodeParams &cp = *reinterpret_cast<cudaGraphNodeParams *>(cp_storage);
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t cond_node;
  SPSS_CUDA_TRY(cudaGraphAddNode(&cond_node, graph, &set_node, nullptr, 1, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  SPSS_CUDA_TRY(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  const unsigned long long before_body = ctx->launches;
  int rc = launch_rebuild(ctx, P);
  g.per_rebuild = (int) (ctx->launches - before_body);
  cudaGraph_t body_out = body;
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &body_out);
  if (rc != SPSS_OK) return rc;
  SPSS_CUDA_TRY(e);
  // nodes 3-4: step and control
  SPSS_CUDA_TRY(cudaStreamBeginCaptureToGraph(ctx->stream, graph, &cond_node, nullptr, 1, cudaStreamCaptureModeRelaxed));
  rc = launch_step(ctx, stepper, P);
  if (rc == SPSS_OK && sampling) rc = launch_sampling(ctx, P, 1);
  e = cudaStreamEndCapture(ctx->stream, &graph);
  if (rc != SPSS_OK) return rc;
  SPSS_CUDA_TRY(e);
  SPSS_CUDA_TRY(cudaGraphInstantiate(&g.exec, graph, 0));
  g.graph = graph;
  g.per_step = (int) (ctx->launches - launches0) - g.per_rebuild;
  g.form = GRAPH_CONDITIONAL;
  ctx->launches = launches0;  // captured, not launched
  return SPSS_OK;
}

// The rebuild as a graph that the control kernel can launch on the device.
static int build_device_rebuild(spss_ctx *ctx, const FastParams &P, GraphEntry &g)
{
  cudaGraph_t rg = nullptr;
  const unsigned long long before = ctx->launches;
  SPSS_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
  const int rc = launch_rebuild(ctx, P);
  const cudaError_t e = cudaStreamEndCapture(ctx->stream, &rg);
  g.per_rebuild = (int) (ctx->launches - before);
  if (rc != SPSS_OK)
  {
    if (rg) cudaGraphDestroy(rg);
    return rc;
  }
  SPSS_CUDA_TRY(e);
  g.rebuild_graph = rg;
  SPSS_CUDA_TRY(cudaGraphInstantiate(&g.rebuild_exec, rg, cudaGraphInstantiateFlagDeviceLaunch));
  SPSS_CUDA_TRY(cudaGraphUpload(g.rebuild_exec, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

// One step as a graph.  Verlet lists (and the trigger of list-less Verlet
// contexts): step and control, the control kernel tail-launching the rebuild
// graph when the trigger fires, so a step without a rebuild is two kernels
// and no conditional node (a conditional node and its set-condition kernel
// cost about 12 us per step on this GB300); the conditional form where this
// device refuses device-launched graphs (or when spss_set_device_rebuild
// asks for it, for every kind).  Cell lists: the rebuild and the step, every
// step.  Kinds without lists: the step alone.
static int build_graph_on(spss_ctx *ctx, int stepper, const FastParams &P, int sampling, GraphEntry &g,
                          unsigned long long launches0)
{
  FastPath *f = ctx->fast;
  const bool trigger = f->kind == KIND_VERLET || f->trigger_only;
  if (trigger && f->device_rebuild)
  {
    const int rc = build_device_rebuild(ctx, P, g);
    if (rc != SPSS_OK)
    {
      // this device or driver refuses device-launched graphs: conditional form
      cudaGetLastError();
      g.release();
      f->device_rebuild = false;
      ctx->launches = launches0;
    }
  }
  if (!f->device_rebuild) return build_graph_conditional(ctx, stepper, P, sampling, g, launches0);
  const unsigned long long launches_step = ctx->launches;
  cudaGraph_t graph = nullptr;
  SPSS_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
  int rc = SPSS_OK;
  if (f->kind == KIND_CELLS)
  {
    f->chain = true;  // binning, re-sort, layout, step and control as one dependent chain
    rc = launch_rebuild(ctx, P);
    g.per_rebuild = 0;
  }
  if (rc == SPSS_OK) rc = launch_step(ctx, stepper, P, trigger ? g.rebuild_exec : nullptr);
  f->chain = false;
  if (rc == SPSS_OK && sampling) rc = launch_sampling(ctx, P, 1);
  const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
  if (rc != SPSS_OK)
  {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  SPSS_CUDA_TRY(e);
  g.graph = graph;
  SPSS_CUDA_TRY(cudaGraphInstantiate(&g.exec, graph, 0));
  g.per_step = (int) (ctx->launches - launches_step);
  g.form = trigger ? GRAPH_DEVICE : (f->kind == KIND_CELLS ? GRAPH_ALWAYS : GRAPH_NONE);
  ctx->launches = launches0;  // captured, not launched
  return SPSS_OK;
}

// nsteps steps: one graph launch each (the first step of a context runs
// eagerly so that every lazily sized buffer exists before capture).
static int run_steps(spss_ctx *ctx, int stepper, double dt, long nsteps, int sampling)
{
  FastPath *f = ctx->fast;
  if (!f->have_state) return SPSS_ERR_INVALID_ARGUMENT;
  if (stepper == SPSS_STEPPER_RK4) return SPSS_ERR_NOT_SUPPORTED;
  if (nsteps <= 0) return nsteps == 0 ? SPSS_OK : SPSS_ERR_INVALID_ARGUMENT;
  if (ctx->timing)
  {
    for (long k = 0; k < nsteps; ++k)
    {
      SPSS_TRY(fast_step(ctx, stepper, 0.0, dt));
      if (sampling) SPSS_TRY(launch_sampling(ctx, params(ctx, dt), 1));
    }
    return sampling ? sync_control(ctx) : SPSS_OK;
  }
  SPSS_TRY(push_host_control(ctx));
  if (!f->binner.offsets.ptr && has_cells(f->kind))
  {
    SPSS_TRY(fast_step(ctx, stepper, 0.0, dt));
    if (sampling) SPSS_TRY(launch_sampling(ctx, params(ctx, dt), 1));
    --nsteps;
    if (nsteps == 0) return sync_control(ctx);
  }
  auto key = std::make_tuple(stepper, dt, sampling ? 1 : 0);
  auto it = f->graphs.find(key);
  if (it == f->graphs.end())
  {
    GraphEntry g;
    SPSS_TRY(build_graph(ctx, stepper, dt, sampling, g));
    it = f->graphs.emplace(key, g).first;
  }
  int rebuilds0 = f->h_ctrl->rebuilds;
  if ((it->second.form == GRAPH_DEVICE || it->second.form == GRAPH_NONE) && f->h_ctrl->rebuild)
  {
    // a rebuild pending before the first step (host request, eager steps):
    // these graphs rebuild only after a step's trigger
    SPSS_TRY(launch_rebuild(ctx, params(ctx, dt)));
    rebuilds0 += 1;
  }
  for (long k = 0; k < nsteps; ++k) SPSS_CUDA_TRY(cudaGraphLaunch(it->second.exec, ctx->stream));
  const int rc = sync_control(ctx);
  ctx->launches += (unsigned long long) nsteps * it->second.per_step
      + (unsigned long long) (f->h_ctrl->rebuilds - rebuilds0) * it->second.per_rebuild;
  return rc;
}

int fast_steps(spss_ctx *ctx, int stepper, double t0, double dt, int nsteps)
{
  (void) t0;
  return run_steps(ctx, stepper, dt, nsteps, 0);
}

int fast_batch_run(spss_ctx *ctx, int stepper, double dt, long nsteps, long sample_every, long sample_from)
{
  FastPath *f = ctx->fast;
  if (sample_every < 0 || sample_from < 0) return SPSS_ERR_INVALID_ARGUMENT;
  f->h_ctrl->sample_every = sample_every;
  f->h_ctrl->sample_from = sample_from;
  SPSS_CUDA_TRY(cudaMemcpyAsync(&f->ctrl->sample_every, &f->h_ctrl->sample_every, 2 * sizeof(long long),
                                cudaMemcpyHostToDevice, ctx->stream));
  return run_steps(ctx, stepper, dt, nsteps, sample_every > 0 ? 1 : 0);
}

int fast_batch_stats(spss_ctx *ctx, double *h_out)
{
  FastPath *f = ctx->fast;
  std::vector<double> raw((size_t) 5 * f->nsys);
  SPSS_CUDA_TRY(cudaMemcpyAsync(raw.data(), f->stats.ptr, sizeof(double) * raw.size(), cudaMemcpyDeviceToHost,
                                ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  for (int r = 0; r < f->nsys; ++r)
  {
    const double *st = &raw[5 * (size_t) r];
    const double c = st[4];
    double *o = h_out + 5 * (size_t) r;
    const double m0 = c > 0 ? st[0] / c : 0.0, m2 = c > 0 ? st[2] / c : 0.0;
    o[0] = m0;
    o[1] = c > 0 ? std::max(0.0, st[1] / c - m0 * m0) : 0.0;
    o[2] = m2;
    o[3] = c > 0 ? std::max(0.0, st[3] / c - m2 * m2) : 0.0;
    o[4] = c;
  }
  return SPSS_OK;
}

int fast_batch_reset_stats(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  SPSS_CUDA_TRY(cudaMemsetAsync(f->stats.ptr, 0, sizeof(double) * 5 * f->nsys, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int fast_system_order_parameters(spss_ctx *ctx, double *h_out)
{
  FastPath *f = ctx->fast;
  if (!f->have_state) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_TRY(launch_sampling(ctx, params(ctx, 0.0), 0));
  SPSS_CUDA_TRY(cudaMemcpyAsync(h_out, f->order_out.ptr, sizeof(double) * 4 * f->nsys, cudaMemcpyDeviceToHost,
                                ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int fast_rebuild_count(spss_ctx *ctx, unsigned long long *count)
{
  SPSS_TRY(sync_control(ctx));
  *count = (unsigned long long) ctx->fast->h_ctrl->rebuilds;
  return SPSS_OK;
}

int fast_num_systems(const spss_ctx *ctx)
{
  return ctx->fast ? ctx->fast->nsys : 1;
}

int fast_system_first(const spss_ctx *ctx, int r)
{
  return ctx->fast->h_sys[r].first;
}

int fast_set_tiling(spss_ctx *ctx, int tile_cells, int persistent)
{
  if (tile_cells < 1 || tile_cells > 4096 || (persistent != 0 && persistent != 1)) return SPSS_ERR_INVALID_ARGUMENT;
  FastPath *f = ctx->fast;
  f->persistent = persistent;
  return set_tiling(ctx, tile_cells);
}

int fast_set_device_rebuild(spss_ctx *ctx, int enabled)
{
  FastPath *f = ctx->fast;
  if (f->device_rebuild == (enabled != 0)) return SPSS_OK;
  f->device_rebuild = enabled != 0;
  for (auto &g : f->graphs) g.second.release();
  f->graphs.clear();
  return SPSS_OK;
}

int fast_get_tiling(spss_ctx *ctx, int *tile_cells, int *persistent)
{
  *tile_cells = ctx->fast->tile_cells;
  *persistent = ctx->fast->persistent;
  return SPSS_OK;
}

template<class T>
static int copy_device(DeviceArray<T> &dst, const T *src, size_t count, cudaStream_t stream)
{
  SPSS_TRY(dst.reserve(count));
  SPSS_CUDA_TRY(cudaMemcpyAsync(dst.ptr, src, sizeof(T) * count, cudaMemcpyDeviceToDevice, stream));
  return SPSS_OK;
}

template<class T>
static int restore_device(T *dst, const DeviceArray<T> &src, size_t count, cudaStream_t stream)
{
  SPSS_CUDA_TRY(cudaMemcpyAsync(dst, src.ptr, sizeof(T) * count, cudaMemcpyDeviceToDevice, stream));
  return SPSS_OK;
}

static int take_snapshot(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  Snapshot &S = f->snap;
  const size_t n = (size_t) ctx->p.n;
  cudaStream_t st = ctx->stream;
  for (int b = 0; b < 2; ++b)
  {
    SPSS_TRY(copy_device(S.rec[b], f->rec[b].ptr, n, st));
    SPSS_TRY(copy_device(S.aux[b], f->aux[b].ptr, n, st));
  }
  SPSS_TRY(copy_device(S.vel, f->vel.ptr, n, st));
  SPSS_TRY(copy_device(S.pid, f->pid.ptr, n, st));
  SPSS_TRY(copy_device(S.inv, f->inv.ptr, n, st));
  SPSS_TRY(copy_device(S.img, f->img.ptr, n, st));
  SPSS_TRY(copy_device(S.turns, f->turns.ptr, n, st));
  SPSS_TRY(copy_device(S.sysctl, f->sysctl.ptr, (size_t) f->nsys, st));
  SPSS_TRY(copy_device(S.ctrl, f->ctrl, 1, st));
  SPSS_CUDA_TRY(cudaStreamSynchronize(st));
  return SPSS_OK;
}

// Back to the snapshot; the lists are rebuilt before the next step.  `keep`:
// the snapshot stays for another restore.
static int restore_snapshot(spss_ctx *ctx, bool keep = false)
{
  FastPath *f = ctx->fast;
  Snapshot &S = f->snap;
  const size_t n = (size_t) ctx->p.n;
  cudaStream_t st = ctx->stream;
  for (int b = 0; b < 2; ++b)
  {
    SPSS_TRY(restore_device(f->rec[b].ptr, S.rec[b], n, st));
    SPSS_TRY(restore_device(f->aux[b].ptr, S.aux[b], n, st));
  }
  SPSS_TRY(restore_device(f->vel.ptr, S.vel, n, st));
  SPSS_TRY(restore_device(f->pid.ptr, S.pid, n, st));
  SPSS_TRY(restore_device(f->inv.ptr, S.inv, n, st));
  SPSS_TRY(restore_device(f->img.ptr, S.img, n, st));
  SPSS_TRY(restore_device(f->turns.ptr, S.turns, n, st));
  SPSS_TRY(restore_device(f->sysctl.ptr, S.sysctl, (size_t) f->nsys, st));
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->h_ctrl, S.ctrl.ptr, sizeof(FastControl), cudaMemcpyDeviceToHost, st));
  SPSS_CUDA_TRY(cudaStreamSynchronize(st));
  f->h_ctrl->rebuild = 1;
  f->h_ctrl->cells_fresh = 0;  // cell ids are not part of the snapshot
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->ctrl, f->h_ctrl, sizeof(FastControl), cudaMemcpyHostToDevice, st));
  SPSS_CUDA_TRY(cudaStreamSynchronize(st));
  ctx->step_counter = f->h_ctrl->step;
  ctx->accumulated_displacement = f->h_ctrl->acc;
  ctx->should_update_lists = 1;
  if (!keep) S.release();
  return SPSS_OK;
}

// Times `steps` steps (graph launches, CUDA events) for every tile width and
// launch form, each from the state the call found, keeps the fastest and
// puts the state back as it was.  The step results do not depend on the
// tiling.
int fast_autotune(spss_ctx *ctx, int stepper, double dt, int steps, double *best_ms)
{
  FastPath *f = ctx->fast;
  if (!f->have_state || steps < 1) return SPSS_ERR_INVALID_ARGUMENT;
  if (stepper == SPSS_STEPPER_RK4) return SPSS_ERR_NOT_SUPPORTED;
  if (!has_cells(f->kind))
  {
    if (best_ms) *best_ms = 0.0;
    return SPSS_OK;
  }
  const int timing = ctx->timing;
  ctx->timing = 0;
  SPSS_TRY(take_snapshot(ctx));
  const int widths[] = {16, 20, 24, 28, 32, 36, 40, 44, 48, 52, 56, 60, 64};
  double best = 1e300;
  int best_w = f->tile_cells, best_p = f->persistent;
  int rc = SPSS_OK;
  for (int w : widths)
    for (int pers = 0; pers <= 1 && rc == SPSS_OK; ++pers)
    {
      // every candidate from the same state: a list rebuild that the trigger
      // calls for inside the timed steps falls on the same step for all of
      // them (results do not depend on the tiling), not on whichever
      // candidate happens to be running when the accumulated displacement
      // reaches the skin
      rc = restore_snapshot(ctx, true);
      if (rc != SPSS_OK) break;
      f->persistent = pers;
      rc = set_tiling(ctx, w);
      if (rc == SPSS_OK) rc = run_steps(ctx, stepper, dt, 2, 0);  // builds the graph, warms up
      if (rc != SPSS_OK) break;
      cudaEventRecord(ctx->ev0, ctx->stream);
      rc = run_steps(ctx, stepper, dt, steps, 0);
      cudaEventRecord(ctx->ev1, ctx->stream);
      if (rc != SPSS_OK) break;
      float ms = 0.0f;
      SPSS_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
      SPSS_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
      if (ms / steps < best)
      {
        best = ms / steps;
        best_w = w;
        best_p = pers;
      }
    }
  f->persistent = best_p;
  const int rc2 = set_tiling(ctx, best_w);
  const int rc3 = restore_snapshot(ctx);
  ctx->timing = timing;
  if (rc != SPSS_OK) return rc;
  if (rc2 != SPSS_OK) return rc2;
  if (rc3 != SPSS_OK) return rc3;
  if (best_ms) *best_ms = best;
  return SPSS_OK;
}

int fast_set_natural_frequencies(spss_ctx *ctx, const double *d_freqs)
{
  FastPath *f = ctx->fast;
  if (f->kind != KIND_GLOBAL) return SPSS_ERR_NOT_SUPPORTED;  // the reference uses them in the global field only
  fast_set_frequencies_kernel<<<blocks_for(ctx->p.n, kTB), kTB, 0, ctx->stream>>>(d_freqs, ctx->p.n, f->nu.ptr);
  ++ctx->launches;
  return check_launch("fast_set_frequencies_kernel");
}

int fast_noise(spss_ctx *ctx, int stepper, unsigned long long step, double *d_out)
{
  const int per = normals_per_particle(ctx->p.model, stepper);
  if (per == 0) return SPSS_OK;
  NoiseKey nk;
  nk.seed = ctx->p.seed;
  nk.replica = ctx->p.replica;
  nk.step = step;
  fast_noise_kernel<<<blocks_for(ctx->p.n, kTB), kTB, 0, ctx->stream>>>(d_out, ctx->p.n, per, nk, ctx->fast->sys.ptr,
                                                                       ctx->fast->sys_of.ptr);
  ++ctx->launches;
  return check_launch("fast_noise_kernel");
}

int fast_evaluate(spss_ctx *, int, const double *, const double *, double *, double, double)
{
  return SPSS_ERR_NOT_SUPPORTED;
}

int fast_complementary_force(spss_ctx *, double *)
{
  return SPSS_ERR_NOT_SUPPORTED;
}

int fast_apply_pbc(spss_ctx *ctx)
{
  fast_pbc_kernel<<<blocks_for(ctx->p.n, kTB), kTB, 0, ctx->stream>>>(ctx->fast->img.ptr, ctx->p.n);
  ++ctx->launches;
  return check_launch("fast_pbc_kernel");
}

}  // namespace spss
