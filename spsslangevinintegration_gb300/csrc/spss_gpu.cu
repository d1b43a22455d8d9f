// C ABI of libspss_gpu.so: context management, host-array entry points and
// the reductions shared by both arithmetic paths.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>

#include "spss_internal.cuh"

namespace spss
{
const char *last_error_text();

// resolve SPSS_VARIANT_DISPATCH as EvaluateRhs does
// (ParticleSystemFirstOrder.cpp:96-111, ParticleSystemSecondOrder.cpp:91-98)
int variant_for(const spss_ctx *ctx, int variant)
{
  return variant_for_params(ctx->p, variant);
}

void derive_lists(const spss_params &p, double &r_min, double &r_max, int &nc, int &nc_verlet)
{
  r_min = p.rho;
  r_max = p.r_max > 0.0 ? p.r_max : p.rho + 0.05;  // ParticleSystemFirstOrderPtr.cpp:97-98
  nc = std::max(1, (int) (1.0 / p.rho));           // ParticleSystemFirstOrder.cpp:37-38
  nc_verlet = p.nc_verlet > 0 ? p.nc_verlet : nc;
}

int variant_for_params(const spss_params &p, int variant)
{
  if (variant != SPSS_VARIANT_DISPATCH) return variant;
  const double rho = p.rho;
  if (p.model == 1)
  {
    if (rho >= M_SQRT1_2) return SPSS_VARIANT_GLOBAL_FIELD;
    if (rho <= 0.25) return SPSS_VARIANT_LINKED_LIST_VERLET;
    if (rho <= 0.5) return SPSS_VARIANT_VERLET;
    return SPSS_VARIANT_ALL_PAIRS;
  }
  return rho <= 0.25 ? SPSS_VARIANT_LINKED_LIST : SPSS_VARIANT_ALL_PAIRS;
}

// CalculateMaxDisplacement's bookkeeping (ParticleSystemFirstOrder.cpp:685-695),
// in host FP64 so the trigger matches the reference bit for bit.
int host_calculate_max_displacement(spss_ctx *ctx, double max2)
{
  ctx->accumulated_displacement += std::sqrt(max2);
  int flag = 0;
  if (ctx->accumulated_displacement > 0.5 * (ctx->r_max - ctx->r_min))
  {
    ctx->accumulated_displacement = 0.0;
    flag = 1;
  }
  ctx->should_update_lists = flag;
  return SPSS_OK;
}

// Phase and velocity-direction order parameters of an AoS state: per-thread
// FP64 sums, block partials, then one block adds the partials in order.
__global__ void order_partials_kernel(const double *__restrict__ x, int n, int s, int model,
                                      double *__restrict__ partials)
{
  __shared__ double sh[4][256];
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int ip = model == 1 ? 2 : 4;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    double sp, cp;
    sincos(x[(long) s * i + ip], &sp, &cp);
    acc[0] += cp;
    acc[1] += sp;
    if (model == 2)
    {
      const double vx = x[(long) s * i + 2], vy = x[(long) s * i + 3];
      const double v = sqrt(vx * vx + vy * vy);
      if (v > 0.0)
      {
        acc[2] += vx / v;
        acc[3] += vy / v;
      }
    }
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

__global__ void order_finish_kernel(const double *__restrict__ partials, int nparts, int n, int model,
                                    double *__restrict__ out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = 0; b < nparts; ++b)
    for (int q = 0; q < 4; ++q) t[q] += partials[4 * b + q];
  const double re = t[0] / n, im = t[1] / n;
  out[0] = sqrt(re * re + im * im);
  out[1] = atan2(im, re);
  if (model == 2)
  {
    const double vre = t[2] / n, vim = t[3] / n;
    out[2] = sqrt(vre * vre + vim * vim);
    out[3] = atan2(vim, vre);
  } else
  {
    out[2] = out[0];
    out[3] = out[1];
  }
}

int order_parameters_aos(spss_ctx *ctx, const double *d_aos, double out[4])
{
  DeviceArray<double> &buf = ctx->scratch_c;
  const int nparts = std::min(1024, (ctx->p.n + 255) / 256);
  SPSS_TRY(buf.reserve(4 * 1024 + 4));
  order_partials_kernel<<<nparts, 256, 0, ctx->stream>>>(d_aos, ctx->p.n, ctx->s, ctx->p.model, buf.ptr);
  ++ctx->launches;
  SPSS_TRY(check_launch("order_partials_kernel"));
  order_finish_kernel<<<1, 32, 0, ctx->stream>>>(buf.ptr, nparts, ctx->p.n, ctx->p.model, buf.ptr + 4 * 1024);
  ++ctx->launches;
  SPSS_TRY(check_launch("order_finish_kernel"));
  SPSS_CUDA_TRY(cudaMemcpyAsync(out, buf.ptr + 4 * 1024, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

// One observer frame from an AoS FP64 state, element by element as the
// reference's observers compute it: the float conversion, then (wrapped) the
// unit-box wrap `x -= floor(x * 1) * 1` and the phase wrap
// `phi -= floor(phi / 2 pi) * 2 pi`, both evaluated in double on the float
// value and rounded back to float (BinaryObserverFirstOrder.cpp:112-117,
// PeriodicBoundaryConditions.cpp:137-145).  Every rounding is explicit.
__global__ void frame_kernel(const double *__restrict__ x, long n, int s, int model, int wrap, float *__restrict__ out)
{
  const long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int ip = model == 1 ? 2 : 4;
  const double two_pi = 6.283185307179586;
  for (int k = 0; k < s; ++k)
  {
    float v = __double2float_rn(x[(long) s * i + k]);
    if (wrap && k < 2)
    {
      const double d = (double) v;
      v = __double2float_rn(__dsub_rn(d, floor(d)));
    } else if (wrap && k == ip)
    {
      const double d = (double) v;
      v = __double2float_rn(__dsub_rn(d, __dmul_rn(floor(__ddiv_rn(d, two_pi)), two_pi)));
    }
    out[(long) s * i + k] = v;
  }
}

__global__ void accumulate_kernel(double *__restrict__ acc, const double *__restrict__ x, long len)
{
  const long q = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (q < len) acc[q] += x[q];
}

// ------------------------------------------------ allocation-free order parameters
//
// Scratch of spss_order_parameters_noalloc: the per-block partial sums of one
// call (kNoallocBlocks blocks x 4 sums, 32 KiB).  It lives in the library's
// module, so every GPU that loads the library holds it until the process
// exits, and every call shares it.  Each call overwrites the partials of all
// blocks it reads, so nothing has to start at zero; calls that overlap on the
// GPU (two streams at once) race on it.
constexpr int kNoallocBlocks = 1024;
static __device__ __align__(256) double g_noalloc_partials[kNoallocBlocks * 4];
constexpr int kNoallocMaxDevices = 64;
static double *g_noalloc_address[kNoallocMaxDevices];
static std::mutex g_noalloc_mutex;

// Device address of the scratch on the current device, looked up once per
// device (host code cannot use the symbol itself: it names a host stand-in).
static int noalloc_scratch(double **out)
{
  int dev = 0;
  SPSS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocMaxDevices) return SPSS_ERR_NOT_SUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_address[dev])
  {
    void *p = nullptr;
    SPSS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_partials));
    g_noalloc_address[dev] = static_cast<double *>(p);
  }
  *out = g_noalloc_address[dev];
  return SPSS_OK;
}

}  // namespace spss

using namespace spss;

static bool is_f64(const spss_ctx *ctx)
{
  return ctx->p.precision == SPSS_PRECISION_F64;
}

static long state_len(const spss_ctx *ctx)
{
  return (long) ctx->p.n * ctx->s;
}

extern "C" {

int spss_version(void)
{
  return 1;
}

const char *spss_error_string(int code)
{
  switch (code)
  {
    case SPSS_OK: return "ok";
    case SPSS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SPSS_ERR_CUDA: return spss::last_error_text();
    case SPSS_ERR_OUT_OF_MEMORY: return "out of device memory";
    case SPSS_ERR_NOT_SUPPORTED: return "not supported by this context";
    case SPSS_ERR_NONFINITE: return "non-finite state";
    case SPSS_ERR_SIZE: return "array length does not match the context";
    default: return "unknown error";
  }
}

int spss_create(const spss_params *params, spss_ctx **out)
{
  if (!params || !out) return SPSS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const spss_params &p = *params;
  if ((p.model != 1 && p.model != 2) || p.n <= 0 || !(p.rho > 0.0) || !std::isfinite(p.rho)) return SPSS_ERR_INVALID_ARGUMENT;
  if (p.precision != SPSS_PRECISION_F64 && p.precision != SPSS_PRECISION_F32) return SPSS_ERR_INVALID_ARGUMENT;
  if (p.variant < SPSS_VARIANT_DISPATCH || p.variant > SPSS_VARIANT_GLOBAL_FIELD) return SPSS_ERR_INVALID_ARGUMENT;
  spss_ctx *ctx = new (std::nothrow) spss_ctx();
  if (!ctx) return SPSS_ERR_OUT_OF_MEMORY;
  ctx->p = p;
  ctx->s = p.model == 1 ? 4 : 6;
  derive_lists(p, ctx->r_min, ctx->r_max, ctx->nc, ctx->nc_verlet);
  ctx->should_update_lists = 1;
  int rc = SPSS_OK;
  if (cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking))
  {
    cudaGetLastError();
    record_cuda_error(e, "creating the context's stream", __FILE__, __LINE__);
    delete ctx;
    return SPSS_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess)
  {
    cudaGetLastError();
    spss_destroy(ctx);
    return SPSS_ERR_CUDA;
  }
  rc = is_f64(ctx) ? f64_create(ctx) : fast_create(ctx);
  if (rc != SPSS_OK)
  {
    spss_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return SPSS_OK;
}

int spss_destroy(spss_ctx *ctx)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->f64) f64_destroy(ctx);
  if (ctx->fast) fast_destroy(ctx);
  ctx->scratch_a.release();
  ctx->scratch_b.release();
  ctx->scratch_c.release();
  ctx->frame_state.release();
  ctx->frame.release();
  ctx->average.release();
  if (ctx->registered_host && ctx->registered_here) cudaHostUnregister(ctx->registered_host);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  cudaGetLastError();
  delete ctx;
  return SPSS_OK;
}

static int upload(spss_ctx *ctx, spss::DeviceArray<double> &dst, const double *src, long len)
{
  SPSS_TRY(dst.reserve(len));
  SPSS_CUDA_TRY(cudaMemcpyAsync(dst.ptr, src, sizeof(double) * len, cudaMemcpyHostToDevice, ctx->stream));
  return SPSS_OK;
}

int spss_set_state(spss_ctx *ctx, const double *state, long len)
{
  if (!ctx || !state) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != state_len(ctx)) return SPSS_ERR_SIZE;
  SPSS_TRY(upload(ctx, ctx->scratch_a, state, len));
  SPSS_TRY(is_f64(ctx) ? f64_set_state(ctx, ctx->scratch_a.ptr) : fast_set_state(ctx, ctx->scratch_a.ptr));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_get_state(spss_ctx *ctx, double *state, long len)
{
  if (!ctx || !state) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != state_len(ctx)) return SPSS_ERR_SIZE;
  SPSS_TRY(ctx->scratch_a.reserve(len));
  SPSS_TRY(is_f64(ctx) ? f64_get_state(ctx, ctx->scratch_a.ptr) : fast_get_state(ctx, ctx->scratch_a.ptr));
  SPSS_CUDA_TRY(cudaMemcpyAsync(state, ctx->scratch_a.ptr, sizeof(double) * len, cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_evaluate_rhs(spss_ctx *ctx, int variant, const double *state, const double *k_prev, double *k_next,
                      double k_coef, double dt)
{
  if (!ctx || !state || !k_prev || !k_next) return SPSS_ERR_INVALID_ARGUMENT;
  const long len = state_len(ctx);
  SPSS_TRY(upload(ctx, ctx->scratch_a, state, len));
  SPSS_TRY(upload(ctx, ctx->scratch_b, k_prev, len));
  SPSS_TRY(upload(ctx, ctx->scratch_c, k_next, len));
  SPSS_TRY(is_f64(ctx) ? f64_evaluate(ctx, variant, ctx->scratch_a.ptr, ctx->scratch_b.ptr, ctx->scratch_c.ptr, k_coef, dt)
                       : fast_evaluate(ctx, variant, ctx->scratch_a.ptr, ctx->scratch_b.ptr, ctx->scratch_c.ptr, k_coef, dt));
  SPSS_CUDA_TRY(cudaMemcpyAsync(k_next, ctx->scratch_c.ptr, sizeof(double) * len, cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_set_higher_order(spss_ctx *ctx, int on)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  ctx->higher_order = on ? 1 : 0;
  return SPSS_OK;
}

int spss_get_complementary_force(spss_ctx *ctx, double *out, long len)
{
  if (!ctx || !out) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != ctx->p.n) return SPSS_ERR_SIZE;
  SPSS_TRY(ctx->scratch_a.reserve(std::max<long>(len, state_len(ctx))));
  SPSS_TRY(is_f64(ctx) ? f64_complementary_force(ctx, ctx->scratch_a.ptr) : fast_complementary_force(ctx, ctx->scratch_a.ptr));
  SPSS_CUDA_TRY(cudaMemcpyAsync(out, ctx->scratch_a.ptr, sizeof(double) * len, cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_set_natural_frequencies(spss_ctx *ctx, const double *freqs, long len)
{
  if (!ctx || !freqs) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != ctx->p.n) return SPSS_ERR_SIZE;
  SPSS_TRY(upload(ctx, ctx->scratch_a, freqs, len));
  SPSS_TRY(is_f64(ctx) ? f64_set_natural_frequencies(ctx, ctx->scratch_a.ptr)
                       : fast_set_natural_frequencies(ctx, ctx->scratch_a.ptr));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_calculate_max_displacement(spss_ctx *ctx, const double *td, long len)
{
  if (!ctx || !td) return SPSS_ERR_INVALID_ARGUMENT;
  if (!ctx->systems.empty()) return SPSS_ERR_NOT_SUPPORTED;  // one trigger per system: kept on the device
  if (len != state_len(ctx)) return SPSS_ERR_SIZE;
  // max_i (dx^2 + dy^2) in host FP64, exactly as ParticleSystemFirstOrder.cpp:672-684
  double max2 = 0.0;
  for (int i = 0; i < ctx->p.n; ++i)
  {
    const double dx = td[(long) ctx->s * i], dy = td[(long) ctx->s * i + 1];
    const double d2 = dx * dx + dy * dy;
    if (max2 < d2) max2 = d2;
  }
  return host_calculate_max_displacement(ctx, max2);
}

int spss_get_verlet_state(spss_ctx *ctx, double *accumulated_displacement, int *should_update_lists,
                          int *uses_verlet_list)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  if (ctx->fast && ctx->stream) SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (accumulated_displacement) *accumulated_displacement = ctx->accumulated_displacement;
  if (should_update_lists) *should_update_lists = ctx->should_update_lists != 0;
  if (uses_verlet_list) *uses_verlet_list = ctx->uses_verlet_list;
  return SPSS_OK;
}

int spss_get_rebuild_count(spss_ctx *ctx, unsigned long long *count)
{
  if (!ctx || !count) return SPSS_ERR_INVALID_ARGUMENT;
  if (is_f64(ctx))
  {
    *count = ctx->list_builds;
    return SPSS_OK;
  }
  return fast_rebuild_count(ctx, count);
}

int spss_set_should_update_lists(spss_ctx *ctx, int flag)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  ctx->should_update_lists = flag ? 1 : 0;
  return SPSS_OK;
}

int spss_get_pre_linked_list(spss_ctx *ctx, int *out, long len)
{
  if (!ctx || !out) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != ctx->p.n) return SPSS_ERR_SIZE;
  if (!is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  int *pll, *off, *mem, *vo, *ve, ncell;
  long vt;
  SPSS_TRY(f64_lists(ctx, &pll, &off, &mem, &ncell, &vo, &ve, &vt));
  if (!pll) return SPSS_ERR_NOT_SUPPORTED;
  SPSS_CUDA_TRY(cudaMemcpyAsync(out, pll, sizeof(int) * len, cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_get_cells(spss_ctx *ctx, int *offsets, long offsets_len, int *members, long members_len, int *ncell_out)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  if (!is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  int *pll, *off, *mem, *vo, *ve, ncell;
  long vt;
  SPSS_TRY(f64_lists(ctx, &pll, &off, &mem, &ncell, &vo, &ve, &vt));
  if (ncell_out) *ncell_out = ncell;
  if (!off) return SPSS_ERR_NOT_SUPPORTED;
  if (offsets)
  {
    if (offsets_len < ncell + 1) return SPSS_ERR_SIZE;
    SPSS_CUDA_TRY(cudaMemcpyAsync(offsets, off, sizeof(int) * (ncell + 1), cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (members)
  {
    if (members_len < ctx->p.n) return SPSS_ERR_SIZE;
    SPSS_CUDA_TRY(cudaMemcpyAsync(members, mem, sizeof(int) * ctx->p.n, cudaMemcpyDeviceToHost, ctx->stream));
  }
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_get_verlet_lists(spss_ctx *ctx, int *offsets, long offsets_len, int *entries, long entries_len, long *total)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  if (!is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  int *pll, *off, *mem, *vo, *ve, ncell;
  long vt;
  SPSS_TRY(f64_lists(ctx, &pll, &off, &mem, &ncell, &vo, &ve, &vt));
  if (total) *total = vt;
  if (!vo) return SPSS_ERR_NOT_SUPPORTED;
  if (offsets)
  {
    if (offsets_len < ctx->p.n + 1) return SPSS_ERR_SIZE;
    SPSS_CUDA_TRY(cudaMemcpyAsync(offsets, vo, sizeof(int) * (ctx->p.n + 1), cudaMemcpyDeviceToHost, ctx->stream));
  }
  if (entries && vt > 0)
  {
    if (entries_len < vt) return SPSS_ERR_SIZE;
    SPSS_CUDA_TRY(cudaMemcpyAsync(entries, ve, sizeof(int) * vt, cudaMemcpyDeviceToHost, ctx->stream));
  }
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

static int check_stepper(const spss_ctx *ctx, int stepper)
{
  if (stepper < SPSS_STEPPER_RK4 || stepper > SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA) return SPSS_ERR_INVALID_ARGUMENT;
  return SPSS_OK;
}

int spss_step(spss_ctx *ctx, int stepper, double t, double dt)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_TRY(check_stepper(ctx, stepper));
  return is_f64(ctx) ? f64_step(ctx, stepper, t, dt) : fast_step(ctx, stepper, t, dt);
}

int spss_steps(spss_ctx *ctx, int stepper, double t0, double dt, int nsteps)
{
  if (!ctx || nsteps < 0) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_TRY(check_stepper(ctx, stepper));
  if (!is_f64(ctx)) return fast_steps(ctx, stepper, t0, dt, nsteps);
  return f64_steps(ctx, stepper, t0, dt, nsteps);
}

int spss_step_host(spss_ctx *ctx, int stepper, double *state, long len, double t, double dt)
{
  if (!ctx || !state) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != state_len(ctx)) return SPSS_ERR_SIZE;
  SPSS_TRY(check_stepper(ctx, stepper));
  const size_t bytes = sizeof(double) * len;
  if (ctx->registered_host != state || ctx->registered_bytes != bytes)
  {
    if (ctx->registered_host && ctx->registered_here) cudaHostUnregister(ctx->registered_host);
    ctx->registered_host = nullptr;
    ctx->registered_device = nullptr;
    ctx->registered_here = false;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, state) == cudaSuccess && attr.type == cudaMemoryTypeHost &&
        attr.devicePointer)
    {
      // already page-locked and mapped (spss_pinned_alloc, cudaHostAlloc): used as it is
      ctx->registered_host = state;
      ctx->registered_bytes = bytes;
      ctx->registered_device = (double *) attr.devicePointer;
    } else if (cudaHostRegister(state, bytes, cudaHostRegisterMapped) == cudaSuccess)
    {
      ctx->registered_host = state;
      ctx->registered_bytes = bytes;
      ctx->registered_here = true;
      void *dp = nullptr;
      if (cudaHostGetDevicePointer(&dp, state, 0) == cudaSuccess) ctx->registered_device = (double *) dp;
      cudaGetLastError();
    } else
    {
      cudaGetLastError();  // pageable copies still work
    }
  }
  // Registered and mapped: the upload kernel reads the caller's array over the
  // host link and the download kernel writes it back, each in one pass that
  // also converts the layout.  Otherwise stage through device memory.
  double *io = ctx->registered_device;
  if (!io)
  {
    SPSS_TRY(ctx->scratch_a.reserve(len));
    SPSS_CUDA_TRY(cudaMemcpyAsync(ctx->scratch_a.ptr, state, bytes, cudaMemcpyHostToDevice, ctx->stream));
  }
  const double *in = io ? io : ctx->scratch_a.ptr;
  double *out = io ? io : ctx->scratch_a.ptr;
  SPSS_TRY(is_f64(ctx) ? f64_set_state(ctx, in) : fast_set_state(ctx, in));
  SPSS_TRY(is_f64(ctx) ? f64_step(ctx, stepper, t, dt) : fast_step(ctx, stepper, t, dt));
  SPSS_TRY(is_f64(ctx) ? f64_get_state(ctx, out) : fast_get_state(ctx, out));
  if (!io) SPSS_CUDA_TRY(cudaMemcpyAsync(state, ctx->scratch_a.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_get_step_counter(spss_ctx *ctx, unsigned long long *counter)
{
  if (!ctx || !counter) return SPSS_ERR_INVALID_ARGUMENT;
  *counter = ctx->step_counter;
  return SPSS_OK;
}

int spss_set_step_counter(spss_ctx *ctx, unsigned long long counter)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  ctx->step_counter = counter;
  return SPSS_OK;
}

int spss_noise(spss_ctx *ctx, int stepper, unsigned long long step, double *out, long len)
{
  if (!ctx || !out) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_TRY(check_stepper(ctx, stepper));
  const long need = (long) ctx->p.n * normals_per_particle(ctx->p.model, stepper);
  if (len != need) return SPSS_ERR_SIZE;
  if (need == 0) return SPSS_OK;
  SPSS_TRY(ctx->scratch_b.reserve(need));
  SPSS_TRY(is_f64(ctx) ? f64_noise(ctx, stepper, step, ctx->scratch_b.ptr) : fast_noise(ctx, stepper, step, ctx->scratch_b.ptr));
  SPSS_CUDA_TRY(cudaMemcpyAsync(out, ctx->scratch_b.ptr, sizeof(double) * need, cudaMemcpyDeviceToHost, ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_apply_pbc(spss_ctx *ctx)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  return is_f64(ctx) ? f64_apply_pbc(ctx) : fast_apply_pbc(ctx);
}

int spss_order_parameters(spss_ctx *ctx, double *out4)
{
  if (!ctx || !out4) return SPSS_ERR_INVALID_ARGUMENT;
  const double *d;
  if (is_f64(ctx))
  {
    SPSS_TRY(f64_state_ptr(ctx, &d));
  } else
  {
    SPSS_TRY(ctx->scratch_a.reserve(state_len(ctx)));
    SPSS_TRY(fast_get_state(ctx, ctx->scratch_a.ptr));
    d = ctx->scratch_a.ptr;
  }
  return order_parameters_aos(ctx, d, out4);
}

int spss_average_accumulate(spss_ctx *ctx)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  const long len = state_len(ctx);
  if (!ctx->average.ptr)
  {
    SPSS_TRY(ctx->average.reserve(len));
    SPSS_CUDA_TRY(cudaMemsetAsync(ctx->average.ptr, 0, sizeof(double) * len, ctx->stream));
  }
  const double *d;
  if (is_f64(ctx))
  {
    SPSS_TRY(f64_state_ptr(ctx, &d));
  } else
  {
    SPSS_TRY(ctx->scratch_a.reserve(len));
    SPSS_TRY(fast_get_state(ctx, ctx->scratch_a.ptr));
    d = ctx->scratch_a.ptr;
  }
  accumulate_kernel<<<(int) ((len + 255) / 256), 256, 0, ctx->stream>>>(ctx->average.ptr, d, len);
  ++ctx->launches;
  SPSS_TRY(check_launch("accumulate_kernel"));
  ++ctx->average_count;
  return SPSS_OK;
}

int spss_average_get(spss_ctx *ctx, double *mean_state, long len, int *count)
{
  if (!ctx || !mean_state) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != state_len(ctx)) return SPSS_ERR_SIZE;
  if (count) *count = ctx->average_count;
  if (!ctx->average.ptr || ctx->average_count == 0)
  {
    std::memset(mean_state, 0, sizeof(double) * len);
    return SPSS_OK;
  }
  SPSS_CUDA_TRY(cudaMemcpyAsync(mean_state, ctx->average.ptr, sizeof(double) * len, cudaMemcpyDeviceToHost,
                                ctx->stream));
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  // AveragingObserver.cpp:62-64: accumulated / number_of_accumulated_steps
  for (long q = 0; q < len; ++q) mean_state[q] /= ctx->average_count;
  return SPSS_OK;
}

int spss_synchronize(spss_ctx *ctx)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return SPSS_OK;
}

int spss_kernel_launches(spss_ctx *ctx, unsigned long long *count)
{
  if (!ctx || !count) return SPSS_ERR_INVALID_ARGUMENT;
  *count = ctx->launches;
  return SPSS_OK;
}

int spss_order_parameters_noalloc(int model, const double *state, long n, double *out4, void *cuda_stream)
{
  if ((model != 1 && model != 2) || !state || !out4) return SPSS_ERR_INVALID_ARGUMENT;
  if (n <= 0 || n > SPSS_NOALLOC_MAX_PARTICLES) return SPSS_ERR_SIZE;
  double *partials = nullptr;
  SPSS_TRY(noalloc_scratch(&partials));
  const int s = model == 1 ? 4 : 6;
  const int nparts = (int) std::min<long>(kNoallocBlocks, (n + 255) / 256);
  cudaStream_t stream = (cudaStream_t) cuda_stream;
  order_partials_kernel<<<nparts, 256, 0, stream>>>(state, (int) n, s, model, partials);
  SPSS_TRY(check_launch("order_partials_kernel"));
  order_finish_kernel<<<1, 32, 0, stream>>>(partials, nparts, (int) n, model, out4);
  return check_launch("order_finish_kernel");
}

int spss_set_stream(spss_ctx *ctx, void *cuda_stream)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ctx->stream = cuda_stream ? (cudaStream_t) cuda_stream : ctx->own_stream;
  return SPSS_OK;
}

int spss_set_timing(spss_ctx *ctx, int on)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  ctx->timing = on ? 1 : 0;
  ctx->timing_ms = 0.0;
  ctx->timing_count = 0;
  return SPSS_OK;
}

int spss_get_timing(spss_ctx *ctx, double *kernel_ms, unsigned long long *timed_launches)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  if (kernel_ms) *kernel_ms = ctx->timing_ms;
  if (timed_launches) *timed_launches = ctx->timing_count;
  return SPSS_OK;
}

// ------------------------------------------------ trajectory frames

int spss_frame_async(spss_ctx *ctx, int mode, float *dst, long len)
{
  if (!ctx || !dst || (mode != SPSS_FRAME_RAW && mode != SPSS_FRAME_WRAPPED)) return SPSS_ERR_INVALID_ARGUMENT;
  if (len != state_len(ctx)) return SPSS_ERR_SIZE;
  const double *aos = nullptr;
  if (is_f64(ctx))
  {
    SPSS_TRY(f64_state_ptr(ctx, &aos));
  } else
  {
    SPSS_TRY(ctx->frame_state.reserve(len));
    SPSS_TRY(fast_get_state(ctx, ctx->frame_state.ptr));
    aos = ctx->frame_state.ptr;
  }
  SPSS_TRY(ctx->frame.reserve(len));
  const long n = ctx->p.n;
  frame_kernel<<<(int) ((n + 255) / 256), 256, 0, ctx->stream>>>(aos, n, ctx->s, ctx->p.model,
                                                                   mode == SPSS_FRAME_WRAPPED ? 1 : 0, ctx->frame.ptr);
  ++ctx->launches;
  SPSS_TRY(check_launch("frame_kernel"));
  SPSS_CUDA_TRY(cudaMemcpyAsync(dst, ctx->frame.ptr, sizeof(float) * len, cudaMemcpyDefault, ctx->stream));
  return SPSS_OK;
}

int spss_pinned_alloc(size_t bytes, void **out)
{
  if (!out || bytes == 0) return SPSS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (cudaMallocHost(out, bytes) != cudaSuccess)
  {
    cudaGetLastError();
    *out = nullptr;
    return SPSS_ERR_OUT_OF_MEMORY;
  }
  return SPSS_OK;
}

int spss_pinned_free(void *p)
{
  if (!p) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_CUDA_TRY(cudaFreeHost(p));
  return SPSS_OK;
}

// ------------------------------------------------ batches of independent systems

int spss_batch_create(const spss_params *systems, int nsys, spss_ctx **out)
{
  if (!systems || !out || nsys < 1) return SPSS_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (nsys > SPSS_MAX_SYSTEMS) return SPSS_ERR_SIZE;
  const spss_params &p0 = systems[0];
  long total = 0;
  for (int r = 0; r < nsys; ++r)
  {
    const spss_params &q = systems[r];
    if ((q.model != 1 && q.model != 2) || q.n <= 0 || !(q.rho > 0.0) || !std::isfinite(q.rho))
      return SPSS_ERR_INVALID_ARGUMENT;
    if (q.model != p0.model || q.flavor != p0.flavor || q.variant != p0.variant || q.precision != p0.precision ||
        q.seed != p0.seed)
      return SPSS_ERR_INVALID_ARGUMENT;
    total += q.n;
  }
  if (p0.precision != SPSS_PRECISION_F32) return SPSS_ERR_NOT_SUPPORTED;  // batches run the GB300 path
  if (total > 0x7fffffffL) return SPSS_ERR_SIZE;
  spss_ctx *ctx = new (std::nothrow) spss_ctx();
  if (!ctx) return SPSS_ERR_OUT_OF_MEMORY;
  ctx->p = p0;
  ctx->p.n = (int) total;
  ctx->systems.assign(systems, systems + nsys);
  ctx->s = p0.model == 1 ? 4 : 6;
  derive_lists(p0, ctx->r_min, ctx->r_max, ctx->nc, ctx->nc_verlet);
  ctx->should_update_lists = 1;
  if (cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking))
  {
    cudaGetLastError();
    record_cuda_error(e, "creating the context's stream", __FILE__, __LINE__);
    delete ctx;
    return SPSS_ERR_CUDA;
  }
  ctx->stream = ctx->own_stream;
  if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess)
  {
    cudaGetLastError();
    spss_destroy(ctx);
    return SPSS_ERR_CUDA;
  }
  const int rc = fast_create(ctx);
  if (rc != SPSS_OK)
  {
    spss_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return SPSS_OK;
}

int spss_batch_size(spss_ctx *ctx, int *nsys, long *first)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  const int ns = is_f64(ctx) ? 1 : fast_num_systems(ctx);
  if (nsys) *nsys = ns;
  if (first)
  {
    for (int r = 0; r < ns; ++r) first[r] = is_f64(ctx) ? 0 : fast_system_first(ctx, r);
    first[ns] = ctx->p.n;
  }
  return SPSS_OK;
}

int spss_batch_order_parameters(spss_ctx *ctx, double *out, long len)
{
  if (!ctx || !out) return SPSS_ERR_INVALID_ARGUMENT;
  if (is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  if (len != 4L * fast_num_systems(ctx)) return SPSS_ERR_SIZE;
  return fast_system_order_parameters(ctx, out);
}

int spss_batch_run(spss_ctx *ctx, int stepper, double t0, double dt, long nsteps, long sample_every, long sample_from)
{
  (void) t0;
  if (!ctx || nsteps < 0) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_TRY(check_stepper(ctx, stepper));
  if (is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  const int rc = fast_batch_run(ctx, stepper, dt, nsteps, sample_every, sample_from);
  return rc;
}

int spss_batch_stats(spss_ctx *ctx, double *out, long len)
{
  if (!ctx || !out) return SPSS_ERR_INVALID_ARGUMENT;
  if (is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  if (len != (long) SPSS_STATS_PER_SYSTEM * fast_num_systems(ctx)) return SPSS_ERR_SIZE;
  return fast_batch_stats(ctx, out);
}

int spss_batch_reset_stats(spss_ctx *ctx)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  if (is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  return fast_batch_reset_stats(ctx);
}

int spss_set_tiling(spss_ctx *ctx, int tile_cells, int persistent)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  if (is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  return fast_set_tiling(ctx, tile_cells, persistent);
}

int spss_get_tiling(spss_ctx *ctx, int *tile_cells, int *persistent)
{
  if (!ctx || !tile_cells || !persistent) return SPSS_ERR_INVALID_ARGUMENT;
  if (is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  return fast_get_tiling(ctx, tile_cells, persistent);
}

int spss_set_device_rebuild(spss_ctx *ctx, int enabled)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  if (is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  return fast_set_device_rebuild(ctx, enabled);
}

int spss_autotune(spss_ctx *ctx, int stepper, double dt, int steps, double *best_ms_per_step)
{
  if (!ctx) return SPSS_ERR_INVALID_ARGUMENT;
  SPSS_TRY(check_stepper(ctx, stepper));
  if (is_f64(ctx)) return SPSS_ERR_NOT_SUPPORTED;
  return fast_autotune(ctx, stepper, dt, steps, best_ms_per_step);
}

}  // extern "C"
