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
//              its inverse; img[n] box crossings; turns[n] 2*pi turns of phase
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
#include <utility>

#include "spss_internal.cuh"

namespace spss
{

constexpr int kTB = 256;

struct FastControl
{
  unsigned long long step;  // Philox step counter of the next stochastic step
  double acc;               // accumulated displacement (FP64)
  int parity;               // current rec/aux buffer
  int rebuild;              // lists (and slot order) rebuilt before the next evaluation
  unsigned int max2_bits;   // max |dr|^2 of the step, FP32 bits (non-negative floats order as ints)
  int overflow;             // largest Verlet count seen beyond capacity (0: none)
  int rebuilds;             // number of rebuilds performed
  int error;                // bit 0: displacement too large for the fixed-point increment
  int uses_verlet;
  int pad;
};

enum Kind
{
  KIND_ALL_PAIRS = 0,
  KIND_CELLS = 1,
  KIND_VERLET = 2
};

struct FastParams
{
  int n, nc, cap, model;
  int kind, always_rebuild, pad0, pad1;
  float v0, xi, xi_r, xi_phi, sigma, ca, sa;
  float rho2_f, band_f, rmax2_f;
  double rho2_d, half_skin;
  float dt, sqdt, half_dt2, half_dt15, inv_sqrt3, b_r, b_phi;
  uint64_t seed;
  uint32_t replica;
};

struct FastBuffers
{
  uint4 *rec0, *rec1;
  uint4 *aux0, *aux1;
  float2 *vel, *vel_tmp;
  unsigned *pid, *pid_tmp, *inv;
  int2 *img, *img_tmp;
  int *turns, *turns_tmp;
  int *cell_of, *cell_sorted;
  const int *cell_off;
  const int *order;
  short *vl;
  int *vl_cnt;
  int *tile_maxcnt;  // longest list of each tile (rows to stage)
  void *tiles;       // TileLayout of every tile, written at rebuild
  FastControl *ctrl;
};

struct GraphEntry
{
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  int per_step = 0;     // kernels of the unconditional part
  int per_rebuild = 0;  // kernels of the conditional rebuild
};

struct FastPath
{
  DeviceArray<uint4> rec[2], aux[2];
  DeviceArray<float2> vel, vel_tmp;
  DeviceArray<unsigned> pid, pid_tmp, inv;
  DeviceArray<int2> img, img_tmp;
  DeviceArray<int> turns, turns_tmp, cell_of, cell_sorted, vl_cnt, tile_maxcnt;
  DeviceArray<short> vl;
  DeviceArray<unsigned char> tiles;
  Binner binner;
  FastControl *ctrl = nullptr;    // device
  FastControl *h_ctrl = nullptr;  // pinned mirror
  int kind = KIND_CELLS;
  int nc_build = 1;
  int cap = 0;
  bool have_state = false;
  bool perm_valid = false;
  std::map<std::pair<int, double>, GraphEntry> graphs;
};

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ uint64_t join64(uint32_t hi, uint32_t lo)
{
  return ((uint64_t) hi << 32) | lo;
}

// round-toward-zero f * 2^64 as a signed integer, exact for the 24-bit
// mantissa; |f| < 0.5 (one step never moves a particle half a box).
__device__ __forceinline__ long long fix64_of(float f, int &err)
{
  const uint32_t b = __float_as_uint(f);
  const int e = (int) ((b >> 23) & 0xffu);
  if (e == 0) return 0;
  if (e >= 126)
  {
    err = 1;
    return 0;
  }
  const long long m = (long long) ((b & 0x7fffffu) | 0x800000u);
  const int sh = e - 86;
  long long v = sh >= 0 ? (m << sh) : (sh > -24 ? (m >> (-sh)) : 0);
  return (b >> 31) ? -v : v;
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

__device__ __forceinline__ void phase_sincos(uint32_t P, float &s, float &c)
{
  sincospif((float) (int) P * 4.656612873077393e-10f, &s, &c);  // P * 2^-31 in [-1, 1)
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
    const double ex = (double) (long long) (join64(rj.x, l.x) - Xi) * 5.421010862427522e-20;
    const double ey = (double) (long long) (join64(rj.y, l.y) - Yi) * 5.421010862427522e-20;
    in = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)) <= P.rho2_d;
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

template<bool OMEGA>
__device__ __forceinline__ void candidate(const FastParams &P, const uint4 &ri, uint64_t Xi, uint64_t Yi,
                                          const uint4 *__restrict__ rec, const uint4 *__restrict__ aux, int j, Acc &a)
{
  const uint4 rj = __ldg(&rec[j]);
  if (in_range(P, ri, Xi, Yi, rj, aux, j)) accumulate(a, rj, OMEGA ? __uint_as_float(__ldg(&aux[j].w)) : 0.0f);
}

// Four list entries at a time: the entry loads, then the record loads, then
// the omega loads of the pairs in range are issued together, so a thread has
// several gathers in flight instead of a chain of dependent ones.
template<bool OMEGA>
__device__ __forceinline__ void candidates4(const FastParams &P, const uint4 &ri, uint64_t Xi, uint64_t Yi,
                                            const uint4 *__restrict__ rec, const uint4 *__restrict__ aux,
                                            const int j[4], Acc &a)
{
  uint4 r[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) r[u] = __ldg(&rec[j[u]]);
  bool in[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) in[u] = in_range(P, ri, Xi, Yi, r[u], aux, j[u]);
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
  B.img[q] = im;
  B.turns[q] = (int) ft;
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
    const int2 im = B.img[q];
    double *st = rows + s * threadIdx.x;
    st[0] = (double) im.x + (double) join64(r.x, a.x) * 5.421010862427522e-20;
    st[1] = (double) im.y + (double) join64(r.y, a.y) * 5.421010862427522e-20;
    const int ip = model == 1 ? 2 : 4;
    st[ip] = 6.283185307179586 * ((double) B.turns[q] + (double) a.z * 2.3283064365386963e-10);
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

__global__ void fast_cells_kernel(FastParams P, FastBuffers B)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.n) return;
  const int par = B.ctrl->parity;
  const uint4 r = (par ? B.rec1 : B.rec0)[q];
  const uint4 a = (par ? B.aux1 : B.aux0)[q];
  B.cell_of[q] = cell_of_fix(join64(r.x, a.x), join64(r.y, a.y), P.nc);
}

// New slot q takes the particle of old slot order[q] (cells contiguous,
// ascending old slot inside a cell).  Writes the other rec/aux buffer.
__global__ void fast_permute_kernel(FastParams P, FastBuffers B)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.n) return;
  const int par = B.ctrl->parity;
  const int src = B.order[q];
  (par ? B.rec0 : B.rec1)[q] = (par ? B.rec1 : B.rec0)[src];
  (par ? B.aux0 : B.aux1)[q] = (par ? B.aux1 : B.aux0)[src];
  const unsigned p = B.pid[src];
  B.pid_tmp[q] = p;
  B.inv[p] = (unsigned) q;
  B.img_tmp[q] = B.img[src];
  B.turns_tmp[q] = B.turns[src];
  if (P.model == 2) B.vel_tmp[q] = B.vel[src];
  B.cell_sorted[q] = B.cell_of[src];
}

__global__ void fast_copyback_kernel(FastParams P, FastBuffers B)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.n) return;
  B.pid[q] = B.pid_tmp[q];
  B.img[q] = B.img_tmp[q];
  B.turns[q] = B.turns_tmp[q];
  if (P.model == 2) B.vel[q] = B.vel_tmp[q];
}

// The permuted state lives in the other buffer; lists are now current.
__global__ void fast_after_rebuild_kernel(FastControl *ctrl, int permuted)
{
  if (permuted) ctrl->parity ^= 1;
  ctrl->rebuild = 0;
  ctrl->rebuilds += 1;
}

// ---------------------------------------------------------------- tiles
//
// A tile is a run of kTileCells cells of one row of the rebuild grid; one CTA
// steps the particles of a tile.  Slots are sorted by cell, so the tile's
// particles are one slot range and the records of its 3 x (kTileCells + 2)
// neighbour cells are at most six slot segments (three rows, each split in
// two where the periodic x-wrap crosses the row end).  The CTA stages those
// segments into shared memory with TMA bulk copies; the Verlet list of a
// particle in a staged tile stores shared-memory indices directly.

constexpr int kTileCells = 32;    // cells per tile
constexpr int kTileCap = 512;     // staged neighbour records per CTA (2 x 8 KiB)
constexpr int kTileThreads = 128;
constexpr long long kWaitCycles = 1ll << 31;  // about one second at the SM clock

struct TileLayout
{
  int p_begin, p_end;  // slots of the tile's own particles
  int nseg, total;     // staged segments (ascending slot order) and records
  int start[6], len[6], base[6];
  int staged;          // the neighbourhood fits kTileCap records
};

__host__ __device__ __forceinline__ int tiles_per_row(int nc)
{
  return (nc + kTileCells - 1) / kTileCells;
}

// Deterministic layout of tile t (the list build and the step compute the same).
__device__ void tile_layout(int t, int nc, const int *__restrict__ off, TileLayout &L)
{
  const int nbx = tiles_per_row(nc);
  const int cy = t / nbx, bx = t - cy * nbx;
  const int cx_lo = bx * kTileCells, cx_hi = min(nc, cx_lo + kTileCells);
  L.p_begin = off[cy * nc + cx_lo];
  L.p_end = off[cy * nc + cx_hi];
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

__device__ __forceinline__ int tile_of_cell(int c, int nc)
{
  const int cy = c / nc;
  return cy * tiles_per_row(nc) + (c - cy * nc) / kTileCells;
}

// Layout of every tile of the rebuild grid, once per rebuild.
__global__ void fast_tile_layout_kernel(FastParams P, FastBuffers B)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.nc * tiles_per_row(P.nc)) return;
  TileLayout L;
  tile_layout(t, P.nc, B.cell_off, L);
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
// the stencil of the rebuild-time cell instead.
__global__ void fast_verlet_build_kernel(FastParams P, FastBuffers B)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P.n) return;
  const int par = B.ctrl->parity;
  const uint4 *rec = par ? B.rec1 : B.rec0;
  const uint4 ri = rec[q];
  const int c = B.cell_sorted[q];
  const int cx = c % P.nc, cy = c / P.nc;
  const int t = tile_of_cell(c, P.nc);
  const TileLayout L = reinterpret_cast<const TileLayout *>(B.tiles)[t];
  int cnt = 0;
  bool far = false;
  const int stride = tile_list_stride(L.p_begin, L.p_end);
  short *lp = B.vl + tile_list_base(P.cap, t, L.p_begin) + (q - L.p_begin);
  for (int sy = -1; sy <= 1; ++sy)
  {
    const int jy = wrap_cell(cy + sy, P.nc);
    for (int sx = -1; sx <= 1; ++sx)
    {
      const int jc = jy * P.nc + wrap_cell(cx + sx, P.nc);
      const int e = B.cell_off[jc + 1];
      for (int j = B.cell_off[jc]; j < e; ++j)
      {
        if (j == q) continue;
        const uint4 rj = __ldg(&rec[j]);
        const float dx = (float) (int) (rj.x - ri.x);
        const float dy = (float) (int) (rj.y - ri.y);
        if (fmaf(dx, dx, dy * dy) <= P.rmax2_f)
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
        candidates4<OMEGA>(P, ri, Xi, Yi, rec, aux, j, a);
      }
      for (; m < cnt; ++m)
      {
        const int j = q + (int) lp[0];
        lp += n;
        candidate<OMEGA>(P, ri, Xi, Yi, rec, aux, j, a);
      }
      return;
    }
    // list unusable: the stencil of the rebuild-time cell holds every particle
    // the list would (displacements since the rebuild < skin / 2)
  }
  if (KIND == KIND_ALL_PAIRS)
  {
    for (int j = 0; j < P.n; ++j)
      if (j != q) candidate<OMEGA>(P, ri, Xi, Yi, rec, aux, j, a);
    return;
  }
  const int c = B.cell_sorted[q];
  const int cx = c % P.nc, cy = c / P.nc;
  // stencil in the reference's order (-1,-1),(0,-1),(1,-1),(-1,0),... (ParticleSystemFirstOrder.cpp:47-52)
  for (int sy = -1; sy <= 1; ++sy)
  {
    const int jy = wrap_cell(cy + sy, P.nc);
    for (int sx = -1; sx <= 1; ++sx)
    {
      const int jc = jy * P.nc + wrap_cell(cx + sx, P.nc);
      const int e = B.cell_off[jc + 1];
      for (int j = B.cell_off[jc]; j < e; ++j)
        if (j != q) candidate<OMEGA>(P, ri, Xi, Yi, rec, aux, j, a);
    }
  }
}

// One staged candidate: the record comes from shared memory; the guard band
// (rare) still reads the slot's low position words from global memory.
template<bool OMEGA>
__device__ __forceinline__ void candidate_staged(const FastParams &P, const uint4 &ri, uint64_t Xi, uint64_t Yi,
                                                 const uint4 *srec, const uint4 *saux, int idx, Acc &a)
{
  const uint4 rj = srec[idx];
  const float dx = (float) (int) (rj.x - ri.x);
  const float dy = (float) (int) (rj.y - ri.y);
  const float d2 = fmaf(dx, dx, dy * dy);
  bool in = d2 <= P.rho2_f;
  if (fabsf(d2 - P.rho2_f) <= P.band_f)
  {
    const uint4 l = saux[idx];
    const double ex = (double) (long long) (join64(rj.x, l.x) - Xi) * 5.421010862427522e-20;
    const double ey = (double) (long long) (join64(rj.y, l.y) - Yi) * 5.421010862427522e-20;
    in = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)) <= P.rho2_d;
  }
  if (in) accumulate(a, rj, OMEGA ? __uint_as_float(saux[idx].w) : 0.0f);
}

// Neighbour sums of slot q from the tile's staged records.
template<int KIND, bool OMEGA>
__device__ __forceinline__ void gather_sums_staged(const FastParams &P, const FastBuffers &B, const uint4 *srec,
                                                   const uint4 *saux, const TileLayout &L,
                                                   const uint4 *__restrict__ rec, const uint4 *__restrict__ aux, int q,
                                                   int cnt, const short *lp, int stride, const uint4 &ri, uint64_t Xi,
                                                   uint64_t Yi, Acc &a)
{
  if (KIND == KIND_VERLET && cnt >= 0)
  {
    const long n = stride;
    int m = 0;
    for (; m + 4 <= cnt; m += 4)
    {
      const int i0 = lp[0], i1 = lp[n], i2 = lp[2 * n], i3 = lp[3 * n];
      lp += 4 * n;
      candidate_staged<OMEGA>(P, ri, Xi, Yi, srec, saux, i0, a);
      candidate_staged<OMEGA>(P, ri, Xi, Yi, srec, saux, i1, a);
      candidate_staged<OMEGA>(P, ri, Xi, Yi, srec, saux, i2, a);
      candidate_staged<OMEGA>(P, ri, Xi, Yi, srec, saux, i3, a);
    }
    for (; m < cnt; ++m)
    {
      candidate_staged<OMEGA>(P, ri, Xi, Yi, srec, saux, lp[0], a);
      lp += n;
    }
    return;
  }
  // cell list, or a Verlet list that did not fit: scan the stencil of the
  // (rebuild-time) cell; each stencil cell is one contiguous staged range
  const int c = B.cell_sorted[q];
  const int cx = c % P.nc, cy = c / P.nc;
  for (int sy = -1; sy <= 1; ++sy)
  {
    const int jy = wrap_cell(cy + sy, P.nc);
    for (int sx = -1; sx <= 1; ++sx)
    {
      const int jc = jy * P.nc + wrap_cell(cx + sx, P.nc);
      const int b = B.cell_off[jc], e = B.cell_off[jc + 1];
      if (e <= b) continue;
      const int i0 = staged_index(L, b);
      if (i0 < 0 || i0 + (e - b) > L.total)
      {
        // not inside the staged segments (cannot happen for a cell of this tile's stencil)
        for (int j = b; j < e; ++j)
          if (j != q) candidate<OMEGA>(P, ri, Xi, Yi, rec, aux, j, a);
        continue;
      }
      const int self = q - b;
      for (int u = 0; u < e - b; ++u)
        if (u != self) candidate_staged<OMEGA>(P, ri, Xi, Yi, srec, saux, i0 + u, a);
    }
  }
}

// Exactly the normals the stepper consumes, in the reference's draw order.
template<int MODEL, int STEPPER>
__device__ __forceinline__ void draw_noise(const FastParams &P, unsigned long long step, unsigned p, float z[6])
{
  constexpr int kNeed = MODEL == 1 ? (STEPPER == 1 ? 1 : 2) : (STEPPER == 1 ? 3 : 6);
  NoiseKey nk;
  nk.seed = P.seed;
  nk.replica = P.replica;
  nk.step = step;
  const uint4 u = philox_block(nk, p, 0);
  box_muller_f32(u.x, u.y, z[0], z[1]);
  if (kNeed > 2) box_muller_f32(u.z, u.w, z[2], z[3]);
  if (kNeed > 4)
  {
    const uint4 u1 = philox_block(nk, p, 1);
    box_muller_f32(u1.x, u1.y, z[4], z[5]);
  }
}

// Derivative from the neighbour sums, SE or SRK update in fixed point, new
// record.  Returns |dr|^2 of the step.
template<int MODEL, int STEPPER>
__device__ __forceinline__ float update_particle(const FastParams &P, const FastBuffers &B, int q, const uint4 &ri,
                                                 const uint4 &ai, float2 v, const Acc &a, const float z[6],
                                                 uint4 *rout, uint4 *aout, int &err)
{
  const uint64_t Xi = join64(ri.x, ai.x), Yi = join64(ri.y, ai.y);
  const float cphi = __uint_as_float(ri.z), sphi = __uint_as_float(ri.w);
  const float wi = __uint_as_float(ai.w);
  // sum sin(phi_j - phi_i - alpha) and sum (omega_j - omega_i) cos(phi_j - phi_i - alpha)
  float f_w = 0.0f, C = 0.0f;  // SE/SRK zero-fill the derivative: an isolated particle keeps 0
  if (a.card > 0)
  {
    const float inv = 1.0f / (float) a.card;
    const float S = cphi * a.ss - sphi * a.sc;  // sum sin(phi_j - phi_i)
    const float K = cphi * a.sc + sphi * a.ss;  // sum cos(phi_j - phi_i)
    f_w = -P.xi_phi * wi + P.sigma * (P.ca * S - P.sa * K) * inv;
    if (STEPPER == 2)
    {
      const float WS = cphi * a.ws - sphi * a.wc;  // sum omega_j sin(phi_j - phi_i)
      const float WK = cphi * a.wc + sphi * a.ws;  // sum omega_j cos(phi_j - phi_i)
      C = P.sigma * inv * ((P.ca * WK + P.sa * WS) - wi * (P.ca * K + P.sa * S));
    }
  }
  const float dt = P.dt;
  float ddx, ddy, dphi, dw;
  if (MODEL == 1)
  {
    const float fx = P.v0 * cphi, fy = P.v0 * sphi, fp = wi;
    if (STEPPER == 1)
    {
      // StochasticEulerStepperPtr.hpp:58-66
      ddx = fx * dt;
      ddy = fy * dt;
      dphi = fp * dt;
      dw = f_w * dt + P.b_phi * (P.sqdt * z[0]);
    } else
    {
      // StochasticRungeKuttaStepperPtr.hpp:54-70
      const float dW = z[0] * P.sqdt;
      const float dZ = P.half_dt15 * (z[0] + P.inv_sqrt3 * z[1]);
      ddx = fx * dt - fp * fy * P.half_dt2;
      ddy = fy * dt + fp * fx * P.half_dt2;
      dphi = fp * dt + f_w * P.half_dt2 + P.b_phi * dZ;
      dw = f_w * dt + (C - P.xi * f_w) * P.half_dt2 + P.b_phi * (dW - P.xi * dZ);
    }
  } else
  {
    const float fvx = -P.xi_r * v.x + P.v0 * cphi, fvy = -P.xi_r * v.y + P.v0 * sphi;
    float dvx, dvy;
    if (STEPPER == 1)
    {
      // StochasticEulerStepper.hpp:44-50 with AddNoise (ParticleSystemSecondOrder.cpp:447-449)
      ddx = dt * v.x;
      ddy = dt * v.y;
      dvx = dt * fvx + P.sqdt * (P.b_r * z[0]);
      dvy = dt * fvy + P.sqdt * (P.b_r * z[1]);
      dphi = dt * wi;
      dw = dt * f_w + P.sqdt * (P.b_phi * z[2]);
    } else
    {
      // second-order strong order 1.5 Taylor scheme (no reference code)
      const float dWx = z[0] * P.sqdt, dZx = P.half_dt15 * (z[0] + P.inv_sqrt3 * z[1]);
      const float dWy = z[2] * P.sqdt, dZy = P.half_dt15 * (z[2] + P.inv_sqrt3 * z[3]);
      const float dWw = z[4] * P.sqdt, dZw = P.half_dt15 * (z[4] + P.inv_sqrt3 * z[5]);
      ddx = v.x * dt + fvx * P.half_dt2 + P.b_r * dZx;
      ddy = v.y * dt + fvy * P.half_dt2 + P.b_r * dZy;
      dvx = fvx * dt + (-P.xi_r * fvx - P.v0 * sphi * wi) * P.half_dt2 + P.b_r * (dWx - P.xi_r * dZx);
      dvy = fvy * dt + (-P.xi_r * fvy + P.v0 * cphi * wi) * P.half_dt2 + P.b_r * (dWy - P.xi_r * dZy);
      dphi = wi * dt + f_w * P.half_dt2 + P.b_phi * dZw;
      dw = f_w * dt + (C - P.xi_phi * f_w) * P.half_dt2 + P.b_phi * (dWw - P.xi_phi * dZw);
    }
    B.vel[q] = make_float2(v.x + dvx, v.y + dvy);
  }
  int cx, cy, ct;
  const uint64_t Xn = advance(Xi, fix64_of(ddx, err), cx);
  const uint64_t Yn = advance(Yi, fix64_of(ddy, err), cy);
  const uint32_t Pn = advance_phase(ai.z, dphi, ct, err);
  float sn, cn;
  phase_sincos(Pn, sn, cn);
  rout[q] = make_uint4((uint32_t) (Xn >> 32), (uint32_t) (Yn >> 32), __float_as_uint(cn), __float_as_uint(sn));
  aout[q] = make_uint4((uint32_t) Xn, (uint32_t) Yn, Pn, __float_as_uint(wi + dw));
  // box crossings and phase turns are rare: read-modify-write only then
  if (cx | cy)
  {
    const int2 im = B.img[q];
    B.img[q] = make_int2(im.x + cx, im.y + cy);
  }
  if (ct) B.turns[q] += ct;
  return fmaf(ddx, ddx, ddy * ddy);
}

// warp max of |dr|^2 for the Verlet trigger; a warp issues its atomic only
// when it can raise the maximum already stored (no block barrier)
__device__ __forceinline__ void publish_max(FastControl *ctrl, float d2max, int err)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) d2max = fmaxf(d2max, __shfl_xor_sync(0xffffffffu, d2max, off));
  err = __any_sync(0xffffffffu, err);
  if ((threadIdx.x & 31) == 0)
  {
    const unsigned bits = __float_as_uint(d2max);
    if (bits > *(volatile unsigned *) &ctrl->max2_bits) atomicMax(&ctrl->max2_bits, bits);
    if (err) atomicOr(&ctrl->error, 1);
  }
}

// One SE or SRK step of one particle per thread, neighbours gathered from
// global memory (all pairs; also usable for every kind).
template<int MODEL, int STEPPER, int KIND>
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
  if (q < P.n)
  {
    const unsigned p = B.pid[q];
    const uint4 ri = rin[q];
    const uint4 ai = ain[q];
    const float2 v = MODEL == 2 ? B.vel[q] : make_float2(0.f, 0.f);
    float z[6];
    draw_noise<MODEL, STEPPER>(P, ctrl->step, p, z);  // overlaps the loads above
    Acc a{0.f, 0.f, 0.f, 0.f, 0};
    gather_sums<KIND, STEPPER == 2>(P, B, rin, ain, q, KIND == KIND_VERLET ? -1 : 0, nullptr, 0, ri,
                                    join64(ri.x, ai.x), join64(ri.y, ai.y), a);
    d2max = update_particle<MODEL, STEPPER>(P, B, q, ri, ai, v, a, z, rout, aout, err);
  }
  publish_max(ctrl, d2max, err);
}

// One SE or SRK step of one tile per CTA with the neighbourhood staged in
// shared memory by TMA bulk copies (cp.async.bulk, completion on an mbarrier).
template<int MODEL, int STEPPER, int KIND>
__global__ void __launch_bounds__(kTileThreads, 8) fast_tile_kernel(FastParams P, FastBuffers B)
{
  __shared__ __align__(16) uint4 srec[kTileCap];
  __shared__ __align__(16) uint4 saux[kTileCap];
  __shared__ __align__(16) short slist[KIND == KIND_VERLET ? kListCap : 8];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ TileLayout L;
  __shared__ int list_staged, list_stride;
  FastControl *ctrl = B.ctrl;
  const int par = ctrl->parity;
  const uint4 *rin = par ? B.rec1 : B.rec0;
  const uint4 *ain = par ? B.aux1 : B.aux0;
  uint4 *rout = par ? B.rec0 : B.rec1;
  uint4 *aout = par ? B.aux0 : B.aux1;
  const short *glist = nullptr;  // this tile's list rows in global memory
  if (threadIdx.x == 0)
  {
    L = reinterpret_cast<const TileLayout *>(B.tiles)[blockIdx.x];
    if (L.p_end <= L.p_begin) L.staged = 0;
    list_stride = tile_list_stride(L.p_begin, L.p_end);
    const int rows = KIND == KIND_VERLET ? B.tile_maxcnt[blockIdx.x] : 0;
    const uint32_t list_bytes = 2u * (uint32_t) rows * (uint32_t) list_stride;
    list_staged = L.staged && KIND == KIND_VERLET && rows > 0 && rows * list_stride <= kListCap;
    if (L.staged)
    {
      const uint32_t mb = smem_u32(&mbar);
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      const uint32_t tx = 32u * L.total + (list_staged ? list_bytes : 0u);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(tx) : "memory");
      for (int k = 0; k < L.nseg; ++k)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(&srec[L.base[k]])),
                     "l"(rin + L.start[k]), "r"(16u * L.len[k]), "r"(mb)
                     : "memory");
      for (int k = 0; k < L.nseg; ++k)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(&saux[L.base[k]])),
                     "l"(ain + L.start[k]), "r"(16u * L.len[k]), "r"(mb)
                     : "memory");
      if (list_staged)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(slist)),
                     "l"(B.vl + tile_list_base(P.cap, blockIdx.x, L.p_begin)), "r"(list_bytes), "r"(mb)
                     : "memory");
    }
  }
  __syncthreads();
  const bool staged = L.staged;
  if (L.p_end <= L.p_begin) return;
  if (KIND == KIND_VERLET) glist = B.vl + tile_list_base(P.cap, blockIdx.x, L.p_begin);
  if (staged)
  {
    // wait for the bulk copies (phase 0), bounded in time
    const uint32_t mb = smem_u32(&mbar);
    uint32_t done = 0;
    long long t0 = clock64();
    while (!done && clock64() - t0 < kWaitCycles)
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
                   : "=r"(done)
                   : "r"(mb)
                   : "memory");
    if (!__syncthreads_and(done))
    {
      // the copies did not complete in time: report, give them a second bounded
      // wait so none is in flight when the CTA exits, and leave this tile
      if (threadIdx.x == 0) atomicOr(&ctrl->error, 2);
      t0 = clock64();
      while (!done && clock64() - t0 < kWaitCycles)
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(mb)
            : "memory");
      return;
    }
  }
  float d2max = 0.0f;
  int err = 0;
  for (int q = L.p_begin + threadIdx.x; q < L.p_end; q += blockDim.x)
  {
    const unsigned p = B.pid[q];
    const uint4 ri = rin[q];
    const uint4 ai = ain[q];
    const int cnt = KIND == KIND_VERLET ? B.vl_cnt[q] : 0;
    const float2 v = MODEL == 2 ? B.vel[q] : make_float2(0.f, 0.f);
    float z[6];
    draw_noise<MODEL, STEPPER>(P, ctrl->step, p, z);
    Acc a{0.f, 0.f, 0.f, 0.f, 0};
    const uint64_t Xi = join64(ri.x, ai.x), Yi = join64(ri.y, ai.y);
    const int i = q - L.p_begin;
    const short *lp = KIND == KIND_VERLET ? (list_staged ? slist + i : glist + i) : nullptr;
    if (staged)
      gather_sums_staged<KIND, STEPPER == 2>(P, B, srec, saux, L, rin, ain, q, cnt, lp, list_stride, ri, Xi, Yi, a);
    else
      gather_sums<KIND, STEPPER == 2>(P, B, rin, ain, q, cnt, lp, list_stride, ri, Xi, Yi, a);
    d2max = fmaxf(d2max, update_particle<MODEL, STEPPER>(P, B, q, ri, ai, v, a, z, rout, aout, err));
  }
  publish_max(ctrl, d2max, err);
}

// After a step: advance the noise counter and the buffer parity, accumulate
// the displacement in FP64 and set the rebuild flag
// (CalculateMaxDisplacement, ParticleSystemFirstOrder.cpp:670-696).
__global__ void fast_control_kernel(FastControl *ctrl, double half_skin, int always_rebuild, int verlet)
{
  ctrl->step += 1;
  ctrl->parity ^= 1;
  const double max2 = (double) __uint_as_float(ctrl->max2_bits);
  ctrl->max2_bits = 0u;
  if (always_rebuild)
  {
    ctrl->rebuild = 1;
    return;
  }
  if (verlet)
  {
    ctrl->acc += sqrt(max2);
    if (ctrl->acc > half_skin)
    {
      ctrl->acc = 0.0;
      ctrl->rebuild = 1;
    }
  }
}

__global__ void fast_set_condition_kernel(const FastControl *ctrl, cudaGraphConditionalHandle handle)
{
  cudaGraphSetConditional(handle, ctrl->rebuild ? 1u : 0u);
}

__global__ void fast_noise_kernel(double *__restrict__ out, int n, int per, NoiseKey nk)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  float z[8];
  normals4_f32(nk, (uint32_t) p, 0, z);
  if (per > 4) normals4_f32(nk, (uint32_t) p, 1, z + 4);
  for (int d = 0; d < per; ++d) out[(long) per * p + d] = (double) z[d];
}

// ApplyPeriodicBoundaryConditions: positions are kept wrapped; forget the box crossings.
__global__ void fast_pbc_kernel(int2 *img, int n)
{
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) img[q] = make_int2(0, 0);
}

// ---------------------------------------------------------------- host side

static int blocks_for(long n, int tb)
{
  return (int) ((n + tb - 1) / tb);
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
  B.img_tmp = f->img_tmp.ptr;
  B.turns = f->turns.ptr;
  B.turns_tmp = f->turns_tmp.ptr;
  B.cell_of = f->cell_of.ptr;
  B.cell_sorted = f->cell_sorted.ptr;
  B.cell_off = f->binner.offsets.ptr;
  B.order = f->binner.members.ptr;
  B.vl = f->vl.ptr;
  B.vl_cnt = f->vl_cnt.ptr;
  B.tile_maxcnt = f->tile_maxcnt.ptr;
  B.tiles = f->tiles.ptr;
  B.ctrl = f->ctrl;
  return B;
}

static FastParams params(spss_ctx *ctx, double dt)
{
  const spss_params &p = ctx->p;
  FastPath *f = ctx->fast;
  FastParams P;
  std::memset(&P, 0, sizeof(P));
  P.n = p.n;
  P.nc = f->nc_build;
  P.cap = f->cap;
  P.model = p.model;
  P.kind = f->kind;
  P.always_rebuild = f->kind == KIND_CELLS ? 1 : 0;
  P.v0 = (float) p.v0;
  P.xi = (float) p.xi;
  P.xi_r = (float) p.xi_r;
  // first order: the torque friction is xi; second order: xi_phi
  P.xi_phi = (float) (p.model == 1 ? p.xi : p.xi_phi);
  P.sigma = (float) p.sigma;
  P.ca = (float) std::cos(p.alpha);
  P.sa = (float) std::sin(p.alpha);
  const double rho2 = p.rho * p.rho;
  P.rho2_d = rho2;
  // FP32 pair distances are squared differences of the 32-bit position words,
  // i.e. in units of 2^-64 of the box area
  const double area = 18446744073709551616.0;
  P.rho2_f = (float) (rho2 * area);
  // |d2_f - d2| <= 2 (|dx| + |dy|) 2^-32 + 2^-32 + 4 d2 2^-24 near r = rho; doubled
  P.band_f = (float) (area * 2.0 * (4.0 * p.rho * 2.3283064365386963e-10 + 2.3283064365386963e-10 + 4.0 * rho2 * 5.9604644775390625e-8));
  const double rmax2 = ctx->r_max * ctx->r_max;
  P.rmax2_f = (float) (area * (rmax2 + 2.0 * (4.0 * ctx->r_max * 2.3283064365386963e-10 + 4.0 * rmax2 * 5.9604644775390625e-8)));
  P.half_skin = 0.5 * (ctx->r_max - ctx->r_min);
  P.dt = (float) dt;
  P.sqdt = (float) std::sqrt(dt);
  P.half_dt2 = (float) (0.5 * dt * dt);
  P.half_dt15 = (float) (0.5 * std::pow(dt, 1.5));
  P.inv_sqrt3 = (float) (1.0 / std::sqrt(3.0));
  P.b_r = (float) std::sqrt(2.0 * p.D_r);
  P.b_phi = (float) std::sqrt(2.0 * p.D_phi);
  P.seed = p.seed;
  P.replica = p.replica;
  return P;
}

int fast_create(spss_ctx *ctx)
{
  FastPath *f = new FastPath();
  ctx->fast = f;
  const spss_params &p = ctx->p;
  const int n = p.n;
  const int variant = variant_for(ctx, p.variant);
  switch (variant)
  {
    case SPSS_VARIANT_ALL_PAIRS:
      f->kind = KIND_ALL_PAIRS;
      f->nc_build = 1;
      break;
    case SPSS_VARIANT_LINKED_LIST:
      f->kind = KIND_CELLS;
      f->nc_build = ctx->nc;
      break;
    case SPSS_VARIANT_VERLET:
      // O(N^2) list build = every pair within r_max: cells no smaller than r_max
      f->kind = KIND_VERLET;
      f->nc_build = std::max(1, (int) (1.0 / ctx->r_max));
      if (f->nc_build < 3) return SPSS_ERR_NOT_SUPPORTED;
      break;
    case SPSS_VARIANT_LINKED_LIST_VERLET:
      f->kind = KIND_VERLET;
      f->nc_build = ctx->nc_verlet;
      break;
    default:
      return SPSS_ERR_NOT_SUPPORTED;  // global field: FP64 contexts
  }
  if (f->kind == KIND_VERLET) ctx->uses_verlet_list = 1;
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
  SPSS_TRY(f->img_tmp.reserve(n));
  SPSS_TRY(f->turns.reserve(n));
  SPSS_TRY(f->turns_tmp.reserve(n));
  SPSS_TRY(f->cell_of.reserve(n));
  SPSS_TRY(f->cell_sorted.reserve(n));
  SPSS_TRY(f->vl_cnt.reserve(n));
  if (f->kind != KIND_ALL_PAIRS)
    SPSS_TRY(f->tiles.reserve(sizeof(TileLayout) * (size_t) f->nc_build * tiles_per_row(f->nc_build)));
  if (f->kind == KIND_VERLET)
  {
    // mean list length: pi r_max^2 n (unit box); room for six standard deviations
    const double lam = M_PI * ctx->r_max * ctx->r_max * n;
    f->cap = std::max(16, ((int) std::ceil(lam + 6.0 * std::sqrt(lam) + 8.0) + 3) & ~3);
    const long ntiles = (long) f->nc_build * tiles_per_row(f->nc_build);
    SPSS_TRY(f->vl.reserve((size_t) f->cap * ((size_t) n + 16 * (size_t) ntiles + 16)));
    SPSS_TRY(f->tile_maxcnt.reserve((size_t) ntiles));
  }
  SPSS_CUDA_TRY(cudaMalloc((void **) &f->ctrl, sizeof(FastControl)));
  SPSS_CUDA_TRY(cudaMallocHost((void **) &f->h_ctrl, sizeof(FastControl)));
  std::memset(f->h_ctrl, 0, sizeof(FastControl));
  f->h_ctrl->rebuild = 1;
  f->h_ctrl->uses_verlet = f->kind == KIND_VERLET;
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->ctrl, f->h_ctrl, sizeof(FastControl), cudaMemcpyHostToDevice, ctx->stream));
  SPSS_CUDA_TRY(cudaMemsetAsync(f->vel.ptr, 0, sizeof(float2) * n, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

void fast_destroy(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  if (!f) return;
  for (auto &g : f->graphs)
  {
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
    if (g.second.graph) cudaGraphDestroy(g.second.graph);
  }
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
  f->img_tmp.release();
  f->turns.release();
  f->turns_tmp.release();
  f->cell_of.release();
  f->cell_sorted.release();
  f->vl.release();
  f->vl_cnt.release();
  f->tile_maxcnt.release();
  f->tiles.release();
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
  if (f->kind != KIND_ALL_PAIRS)
  {
    fast_cells_kernel<<<blocks_for(n, kTB), kTB, 0, ctx->stream>>>(P, B);
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_cells_kernel"));
    SPSS_TRY(f->binner.run(f->cell_of.ptr, n, P.nc * P.nc, ctx->stream, ctx->launches));
    const FastBuffers B2 = buffers(ctx);  // binner buffers exist now
    fast_permute_kernel<<<blocks_for(n, kTB), kTB, 0, ctx->stream>>>(P, B2);
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_permute_kernel"));
    fast_copyback_kernel<<<blocks_for(n, kTB), kTB, 0, ctx->stream>>>(P, B2);
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_copyback_kernel"));
  }
  fast_after_rebuild_kernel<<<1, 1, 0, ctx->stream>>>(f->ctrl, f->kind != KIND_ALL_PAIRS);
  ++ctx->launches;
  SPSS_TRY(check_launch("fast_after_rebuild_kernel"));
  if (f->kind != KIND_ALL_PAIRS)
  {
    const int ntiles = P.nc * tiles_per_row(P.nc);
    fast_tile_layout_kernel<<<blocks_for(ntiles, 128), 128, 0, ctx->stream>>>(P, buffers(ctx));
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_tile_layout_kernel"));
  }
  if (f->kind == KIND_VERLET)
  {
    SPSS_CUDA_TRY(cudaMemsetAsync(f->tile_maxcnt.ptr, 0, sizeof(int) * f->tile_maxcnt.count, ctx->stream));
    fast_verlet_build_kernel<<<blocks_for(n, 128), 128, 0, ctx->stream>>>(P, buffers(ctx));
    ++ctx->launches;
    SPSS_TRY(check_launch("fast_verlet_build_kernel"));
  }
  return SPSS_OK;
}

template<int MODEL, int STEPPER>
static void launch_step_kind(spss_ctx *ctx, const FastParams &P, const FastBuffers &B)
{
  const int grid = blocks_for(P.n, kTB);
  const int tiles = P.nc * tiles_per_row(P.nc);
  switch (ctx->fast->kind)
  {
    case KIND_ALL_PAIRS: fast_step_kernel<MODEL, STEPPER, KIND_ALL_PAIRS><<<grid, kTB, 0, ctx->stream>>>(P, B); break;
    case KIND_CELLS:
      fast_tile_kernel<MODEL, STEPPER, KIND_CELLS><<<tiles, kTileThreads, 0, ctx->stream>>>(P, B);
      break;
    default: fast_tile_kernel<MODEL, STEPPER, KIND_VERLET><<<tiles, kTileThreads, 0, ctx->stream>>>(P, B); break;
  }
}

static int launch_step(spss_ctx *ctx, int stepper, const FastParams &P)
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
  fast_control_kernel<<<1, 1, 0, ctx->stream>>>(ctx->fast->ctrl, P.half_skin, P.always_rebuild,
                                                 ctx->fast->kind == KIND_VERLET);
  ++ctx->launches;
  return check_launch("fast_control_kernel");
}

static int sync_control(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  SPSS_CUDA_TRY(cudaMemcpyAsync(f->h_ctrl, f->ctrl, sizeof(FastControl), cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ctx->step_counter = f->h_ctrl->step;
  ctx->accumulated_displacement = f->h_ctrl->acc;
  ctx->should_update_lists = f->h_ctrl->rebuild;
  if (f->h_ctrl->error) return SPSS_ERR_NONFINITE;
  return SPSS_OK;
}

// The host-side step counter and list flag (spss_set_step_counter,
// spss_set_should_update_lists) win over the device copy.
static int push_host_control(spss_ctx *ctx)
{
  FastPath *f = ctx->fast;
  if (f->h_ctrl->step == ctx->step_counter && f->h_ctrl->rebuild == ctx->should_update_lists) return SPSS_OK;
  f->h_ctrl->step = ctx->step_counter;
  f->h_ctrl->rebuild = ctx->should_update_lists;
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

static int build_graph_on(spss_ctx *ctx, int stepper, const FastParams &P, GraphEntry &g,
                          unsigned long long launches0);

// One step as a graph: rebuild under a conditional node, then step + control.
static int build_graph(spss_ctx *ctx, int stepper, double dt, GraphEntry &g)
{
  const FastParams P = params(ctx, dt);
  const unsigned long long launches0 = ctx->launches;
  const int timing = ctx->timing;
  cudaStream_t work = ctx->stream;
  ctx->timing = 0;
  ctx->stream = ctx->own_stream;  // capture needs a non-legacy stream
  int rc_all = build_graph_on(ctx, stepper, P, g, launches0);
  ctx->stream = work;
  ctx->timing = timing;
  return rc_all;
}

static int build_graph_on(spss_ctx *ctx, int stepper, const FastParams &P, GraphEntry &g,
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
  e = cudaStreamEndCapture(ctx->stream, &graph);
  if (rc != SPSS_OK) return rc;
  SPSS_CUDA_TRY(e);
  SPSS_CUDA_TRY(cudaGraphInstantiate(&g.exec, graph, 0));
  g.graph = graph;
  g.per_step = (int) (ctx->launches - launches0) - g.per_rebuild;
  ctx->launches = launches0;  // captured, not launched
  return SPSS_OK;
}

int fast_steps(spss_ctx *ctx, int stepper, double t0, double dt, int nsteps)
{
  (void) t0;
  FastPath *f = ctx->fast;
  if (!f->have_state) return SPSS_ERR_INVALID_ARGUMENT;
  if (stepper == SPSS_STEPPER_RK4) return SPSS_ERR_NOT_SUPPORTED;
  if (nsteps == 0) return SPSS_OK;
  if (ctx->timing)
  {
    for (int k = 0; k < nsteps; ++k) SPSS_TRY(fast_step(ctx, stepper, t0 + (k + 1) * dt, dt));
    return SPSS_OK;
  }
  SPSS_TRY(push_host_control(ctx));
  // the first step runs eagerly so every lazily sized buffer exists before capture
  if (!f->binner.offsets.ptr && f->kind != KIND_ALL_PAIRS)
  {
    SPSS_TRY(fast_step(ctx, stepper, t0 + dt, dt));
    --nsteps;
    if (nsteps == 0) return SPSS_OK;
  }
  auto key = std::make_pair(stepper, dt);
  auto it = f->graphs.find(key);
  if (it == f->graphs.end())
  {
    GraphEntry g;
    SPSS_TRY(build_graph(ctx, stepper, dt, g));
    it = f->graphs.emplace(key, g).first;
  }
  const int rebuilds0 = f->h_ctrl->rebuilds;
  for (int k = 0; k < nsteps; ++k) SPSS_CUDA_TRY(cudaGraphLaunch(it->second.exec, ctx->stream));
  const int rc = sync_control(ctx);
  ctx->launches += (unsigned long long) nsteps * it->second.per_step
      + (unsigned long long) (f->h_ctrl->rebuilds - rebuilds0) * it->second.per_rebuild;
  return rc;
}

int fast_noise(spss_ctx *ctx, int stepper, unsigned long long step, double *d_out)
{
  const int per = normals_per_particle(ctx->p.model, stepper);
  if (per == 0) return SPSS_OK;
  NoiseKey nk;
  nk.seed = ctx->p.seed;
  nk.replica = ctx->p.replica;
  nk.step = step;
  fast_noise_kernel<<<blocks_for(ctx->p.n, kTB), kTB, 0, ctx->stream>>>(d_out, ctx->p.n, per, nk);
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
