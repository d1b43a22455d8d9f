// Internal declarations shared by the translation units of libspss_gpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <vector>

#include "spss_gpu.h"

namespace spss
{

// ------------------------------------------------------------------ errors

struct Status
{
  int code = SPSS_OK;
};

#define SPSS_CUDA_TRY(expr)                                  \
  do                                                         \
  {                                                          \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess)                                   \
    {                                                        \
      ::spss::record_cuda_error(_e, #expr, __FILE__, __LINE__); \
      return SPSS_ERR_CUDA;                                  \
    }                                                        \
  } while (0)

#define SPSS_TRY(expr)          \
  do                            \
  {                             \
    int _rc = (expr);           \
    if (_rc != SPSS_OK) return _rc; \
  } while (0)

void record_cuda_error(cudaError_t e, const char *what, const char *file, int line);
int check_launch(const char *what);

// Programmatic dependent launch along the kernel chain of a cell-list step
// graph.  Every kernel that may be launched with the programmatic attribute
// begins with pdl_enter(): it waits until the kernel before it in the stream
// has completed and its writes are visible (without the attribute the
// instruction does nothing).  No kernel triggers its dependents early: with
// the trigger at the start of every CTA the large cell-list steps ran about
// 2 % slower (N = 4,194,304: 0.6095 -> 0.6204 ms), without it they gained
// (0.6059 ms; N = 65,536: 0.0475 -> 0.0437 ms).
__device__ __forceinline__ void pdl_enter()
{
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// A kernel launch, with the programmatic-serialization attribute when `chained`
// (the kernel must begin with pdl_enter()).
template<typename... Params, typename... Args>
inline cudaError_t launch_chained(bool chained, void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem,
                                  cudaStream_t stream, Args... args)
{
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr.val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = chained ? &attr : nullptr;
  cfg.numAttrs = chained ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// ------------------------------------------------------------------ Philox

// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11).  Counter = (particle, step lo, step hi,
// replica << 8 | block), key = seed.
struct Philox
{
  __host__ __device__ static inline uint4 generate(uint4 c, uint2 k)
  {
#pragma unroll
    for (int r = 0; r < 10; ++r)
    {
      const uint64_t p0 = (uint64_t) 0xD2511F53u * c.x;
      const uint64_t p1 = (uint64_t) 0xCD9E8D57u * c.z;
      const uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
      const uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
      c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
      k.x += 0x9E3779B9u;
      k.y += 0xBB67AE85u;
    }
    return c;
  }
};

// The ten round keys of a seed (the Weyl sequence of Philox4x32-10).
__host__ __device__ inline void philox_round_keys(uint64_t seed, uint32_t kx[10], uint32_t ky[10])
{
  uint32_t a = (uint32_t) seed, b = (uint32_t) (seed >> 32);
  for (int r = 0; r < 10; ++r)
  {
    kx[r] = a;
    ky[r] = b;
    a += 0x9E3779B9u;
    b += 0xBB67AE85u;
  }
}

// Philox4x32-10 with the round keys given (equal to Philox::generate with
// the seed they come from), so a kernel takes them from its parameters
// instead of recomputing the key schedule per draw.
__device__ __forceinline__ uint4 philox_keyed(uint4 c, const uint32_t kx[10], const uint32_t ky[10])
{
#pragma unroll
  for (int r = 0; r < 10; ++r)
  {
    const uint64_t p0 = (uint64_t) 0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t) 0xCD9E8D57u * c.z;
    const uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
    const uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
    c = make_uint4(hi1 ^ c.y ^ kx[r], lo1, hi0 ^ c.w ^ ky[r], lo0);
  }
  return c;
}

struct NoiseKey
{
  uint64_t seed;
  uint32_t replica;
  uint64_t step;
};

__device__ __forceinline__ uint4 philox_block(const NoiseKey &nk, uint32_t particle, uint32_t block)
{
  uint4 c = make_uint4(particle, (uint32_t) nk.step, (uint32_t) (nk.step >> 32), (nk.replica << 8) | block);
  return Philox::generate(c, make_uint2((uint32_t) nk.seed, (uint32_t) (nk.seed >> 32)));
}

// Box-Muller on two 32-bit uniforms in (0, 1): FP64 variant for the
// reference-arithmetic path, FP32 variant for the fast path.
__device__ __forceinline__ void box_muller_f64(uint32_t a, uint32_t b, double &z0, double &z1)
{
  const double u1 = ((double) a + 0.5) * 2.3283064365386963e-10;
  const double u2 = ((double) b + 0.5) * 2.3283064365386963e-10;
  const double r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  z0 = r * c;
  z1 = r * s;
}

// The angle is uniform on (-pi, pi) and goes through the hardware sine and
// cosine (absolute error below 2^-21 there); the radius uses the hardware
// logarithm (absolute error below 2^-21.4 on [0.5, 2], where u1 lies unless the
// radius exceeds 1.18, and 3 ulp beyond): the radius r is off by at most about
// 2^-21.4 / r, more than 1 % relative only for r < 6e-3, which a fraction 2e-5
// of the draws reach, far beneath any statistical resolution of the runs.
// spss_noise evaluates the same function, so replayed noise is bit-identical.
// Rounding is spelled out (__fmul_rn, __fadd_rn) so every inlined copy of this
// function produces the same bits.
__device__ __forceinline__ void box_muller_f32(uint32_t a, uint32_t b, float &z0, float &z1)
{
  const float u1 = __fmul_rn(__fadd_rn((float) (a >> 8), 0.5f), 5.9604644775390625e-8f);
  const float theta = __fmul_rn(__fadd_rn(__fmul_rn((float) (b >> 8), 5.9604644775390625e-8f), -0.49999997f),
                                6.2831853f);
  const float r = sqrtf(__fmul_rn(-2.0f, __logf(u1)));
  float s, c;
  __sincosf(theta, &s, &c);
  z0 = __fmul_rn(r, c);
  z1 = __fmul_rn(r, s);
}

// Six normals from one Philox block (128 bits), for the steps that need six
// (second-order SRK): three Box-Muller pairs with 24-bit radius uniforms (the
// top 24 bits of words 0..2) and 16-bit angle uniforms (the two halves of
// word 3, and the low bytes of words 0 and 1).  A 16-bit angle is resolved to
// 1e-4 rad; the radius keeps the tails of the 24-bit draws above.
__device__ __forceinline__ void box_muller6_f32(const uint4 &u, float z[6])
{
  const uint32_t a[3] = {u.x >> 8, u.y >> 8, u.z >> 8};
  const uint32_t b[3] = {u.w & 0xffffu, u.w >> 16, (u.x & 0xffu) | ((u.y & 0xffu) << 8)};
#pragma unroll
  for (int k = 0; k < 3; ++k)
  {
    const float u1 = __fmul_rn(__fadd_rn((float) a[k], 0.5f), 5.9604644775390625e-8f);
    const float theta = __fmul_rn(__fadd_rn(__fmul_rn(__fadd_rn((float) b[k], 0.5f), 1.52587890625e-5f), -0.5f),
                                  6.2831853f);
    const float r = sqrtf(__fmul_rn(-2.0f, __logf(u1)));
    float s, c;
    __sincosf(theta, &s, &c);
    z[2 * k] = __fmul_rn(r, c);
    z[2 * k + 1] = __fmul_rn(r, s);
  }
}

__device__ __forceinline__ void normals4_f32(const NoiseKey &nk, uint32_t particle, uint32_t block, float z[4])
{
  const uint4 u = philox_block(nk, particle, block);
  box_muller_f32(u.x, u.y, z[0], z[1]);
  box_muller_f32(u.z, u.w, z[2], z[3]);
}

__device__ __forceinline__ void normals4_f64(const NoiseKey &nk, uint32_t particle, uint32_t block, double z[4])
{
  const uint4 u = philox_block(nk, particle, block);
  box_muller_f64(u.x, u.y, z[0], z[1]);
  box_muller_f64(u.z, u.w, z[2], z[3]);
}

inline int normals_per_particle(int model, int stepper)
{
  if (stepper == SPSS_STEPPER_RK4) return 0;
  if (stepper == SPSS_STEPPER_STOCHASTIC_EULER) return model == 1 ? 1 : 3;
  return model == 1 ? 2 : 6;
}

// ------------------------------------------------------------------ device memory

template<class T>
struct DeviceArray
{
  T *ptr = nullptr;
  size_t count = 0;
  int reserve(size_t n)
  {
    if (n <= count && ptr) return SPSS_OK;
    release();
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **) &ptr, n * sizeof(T));
    if (e != cudaSuccess)
    {
      ptr = nullptr;
      count = 0;
      cudaGetLastError();
      return SPSS_ERR_OUT_OF_MEMORY;
    }
    count = n;
    return SPSS_OK;
  }
  void release()
  {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
  }
  size_t bytes() const { return count * sizeof(T); }
};

// Exclusive prefix sum of `n` int32 counts into offsets[0..n] (offsets[n] =
// total), three-phase with recursion on the block sums.
struct Scanner
{
  std::vector<DeviceArray<int>> levels;
  int run(const int *in, int *out, int n, cudaStream_t stream, unsigned long long &launches, bool chained = false);
  int run_level(const int *in, int *out, int n, size_t level, cudaStream_t stream, unsigned long long &launches,
                bool chained);
  void release()
  {
    for (auto &l : levels) l.release();
    levels.clear();
  }
};

// Stable cell binning: cell id per element -> CSR offsets and members that list
// each cell's elements in ascending element order (the push_back order of the
// reference's linked_list_, ParticleSystemFirstOrder.cpp:285-288).
struct Binner
{
  DeviceArray<int> count, offsets, slot, members;
  Scanner scanner;
  int ncell = 0;
  // chained: launches after the first with the programmatic attribute
  int run(const int *cell_of, int n, int ncell, cudaStream_t stream, unsigned long long &launches,
          bool chained = false);
  void release()
  {
    count.release();
    offsets.release();
    slot.release();
    members.release();
    scanner.release();
  }
};

// ------------------------------------------------------------------ contexts

struct F64Path;
struct FastPath;

}  // namespace spss

struct spss_ctx
{
  spss_params p{};  // a batch: the first system's parameters, n = all particles
  std::vector<spss_params> systems;  // a batch: every system (empty for one system)
  int s = 4;
  cudaStream_t stream = nullptr;      // where work is issued
  cudaStream_t own_stream = nullptr;  // created with the context; graph capture runs here
  // CUDA-event timing of the pair-and-update kernel (spss_set_timing)
  int timing = 0;
  double timing_ms = 0.0;
  unsigned long long timing_count = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  unsigned long long launches = 0;
  unsigned long long step_counter = 0;
  int higher_order = 0;
  // Verlet bookkeeping (CalculateMaxDisplacement), kept on the host in FP64.
  double accumulated_displacement = 0.0;
  int should_update_lists = 1;
  int uses_verlet_list = 0;
  unsigned long long list_builds = 0;  // Verlet / cell list builds so far (FP64 path; the fast path counts on the device)
  double r_min = 0.0, r_max = 0.0;
  int nc = 1, nc_verlet = 1;
  // host registration of the caller's array for spss_step_host
  void *registered_host = nullptr;
  size_t registered_bytes = 0;
  double *registered_device = nullptr;  // device view of the registered array (mapped pinned memory)
  bool registered_here = false;         // registered by this context (else the caller's page-locked memory)
  spss::F64Path *f64 = nullptr;
  spss::FastPath *fast = nullptr;
  // AveragingObserver accumulator (FP64, AoS) and its count
  spss::DeviceArray<double> average;
  int average_count = 0;
  // AoS staging buffers for host-array entry points
  spss::DeviceArray<double> scratch_a, scratch_b, scratch_c;
  // trajectory frames (spss_frame_async): the AoS state of a fast context and the float frame
  spss::DeviceArray<double> frame_state;
  spss::DeviceArray<float> frame;
};

namespace spss
{
// F64 (reference arithmetic) path, f64_path.cu
int f64_create(spss_ctx *ctx);
void f64_destroy(spss_ctx *ctx);
int f64_set_state(spss_ctx *ctx, const double *d_aos);
int f64_get_state(spss_ctx *ctx, double *d_aos);
int f64_evaluate(spss_ctx *ctx, int variant, const double *d_state, const double *d_kprev, double *d_knext,
                 double k_coef, double dt);
int f64_step(spss_ctx *ctx, int stepper, double t, double dt);
int f64_steps(spss_ctx *ctx, int stepper, double t0, double dt, int nsteps);
int f64_noise(spss_ctx *ctx, int stepper, unsigned long long step, double *d_out);
int f64_max_displacement(spss_ctx *ctx, const double *d_td, double *max2_out);
int f64_complementary_force(spss_ctx *ctx, double *d_out);
int f64_set_natural_frequencies(spss_ctx *ctx, const double *d_freqs);
int f64_lists(spss_ctx *ctx, int **pll, int **cell_off, int **cell_mem, int *ncell, int **vl_off, int **vl_ent,
              long *vl_total);
int f64_apply_pbc(spss_ctx *ctx);
int f64_state_ptr(spss_ctx *ctx, const double **d_aos);

// Fast (GB300) path, fast_path.cu
int fast_create(spss_ctx *ctx);
void fast_destroy(spss_ctx *ctx);
int fast_rebuild_count(spss_ctx *ctx, unsigned long long *count);
int fast_set_state(spss_ctx *ctx, const double *d_aos);
int fast_get_state(spss_ctx *ctx, double *d_aos);
int fast_evaluate(spss_ctx *ctx, int variant, const double *d_state, const double *d_kprev, double *d_knext,
                  double k_coef, double dt);
int fast_step(spss_ctx *ctx, int stepper, double t, double dt);
int fast_steps(spss_ctx *ctx, int stepper, double t0, double dt, int nsteps);
int fast_noise(spss_ctx *ctx, int stepper, unsigned long long step, double *d_out);
int fast_set_natural_frequencies(spss_ctx *ctx, const double *d_freqs);
int fast_complementary_force(spss_ctx *ctx, double *d_out);
int fast_apply_pbc(spss_ctx *ctx);

int fast_set_tiling(spss_ctx *ctx, int tile_cells, int persistent);
int fast_get_tiling(spss_ctx *ctx, int *tile_cells, int *persistent);
int fast_set_device_rebuild(spss_ctx *ctx, int enabled);
int fast_autotune(spss_ctx *ctx, int stepper, double dt, int steps, double *best_ms);
int fast_system_order_parameters(spss_ctx *ctx, double *h_out);
int fast_batch_run(spss_ctx *ctx, int stepper, double dt, long nsteps, long sample_every, long sample_from);
int fast_batch_stats(spss_ctx *ctx, double *h_out);
int fast_batch_reset_stats(spss_ctx *ctx);
int fast_num_systems(const spss_ctx *ctx);
int fast_system_first(const spss_ctx *ctx, int r);

// Shared helpers, spss_gpu.cu
int order_parameters_aos(spss_ctx *ctx, const double *d_aos, double out[4]);
int host_calculate_max_displacement(spss_ctx *ctx, double max2);
int variant_for(const spss_ctx *ctx, int variant);
int variant_for_params(const spss_params &p, int variant);
// List geometry of a system: r_min = rho, r_max (Verlet cutoff), the cell grid
// of the linked list and of the Verlet rebuild.
void derive_lists(const spss_params &p, double &r_min, double &r_max, int &nc, int &nc_verlet);
}  // namespace spss
