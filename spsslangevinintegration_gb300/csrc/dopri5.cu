// Adaptive Dormand-Prince 5(4) integration with dense output over the FP64
// right-hand side, for the reference's odeint path
// (SimulationEngineFirstOrder.cpp:158-165: integrate_const(make_dense_output(
// eps_abs, eps_rel, runge_kutta_dopri5), system, state, t0, t1, dt, observer)).
// Boost.Odeint is not part of the reference tree and its version is not
// pinned, so this restates the published method, not Boost's code:
//   * the Dormand-Prince tableau (Dormand & Prince, J. Comput. Appl. Math. 6, 1980),
//     first-same-as-last;
//   * the error of a step: max_i |x_err_i| / (eps_abs + eps_rel (|x_i| + h |x'_i|)),
//     x and x' at the start of the step, and the step-size rule: reject if the
//     error exceeds 1 and shrink h by max(0.9 err^(-1/3), 0.2); after an
//     accepted step with error below 0.5 grow h by 0.9 max(err, 5^-5)^(-1/5)
//     (odeint's default error checker and step adjuster, as documented);
//   * dense output by the continuous extension of Hairer, Norsett & Wanner
//     (Solving ODE I, section II.6), evaluated at every observer time.
// The state and every stage stay on the GPU; each step reads one error norm.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "spss_internal.cuh"

namespace spss
{
namespace
{

// Butcher tableau
constexpr double kC[7] = {0.0, 1.0 / 5.0, 3.0 / 10.0, 4.0 / 5.0, 8.0 / 9.0, 1.0, 1.0};
constexpr double kA[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {1.0 / 5.0, 0, 0, 0, 0, 0},
    {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
    {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0},
    {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0},
    {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0},
    {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}};
// fifth-order weights minus fourth-order weights (the error estimate), stages 1..7
constexpr double kE[7] = {71.0 / 57600.0,      0.0, -71.0 / 16695.0, 71.0 / 1920.0,
                          -17253.0 / 339200.0, 22.0 / 525.0, -1.0 / 40.0};
// dense-output coefficients of the continuous extension
constexpr double kD[7] = {-12715105075.0 / 11282082432.0, 0.0, 87487479700.0 / 32700410799.0,
                          -10690763975.0 / 1880347072.0,  701980252875.0 / 199316789632.0,
                          -1453857185.0 / 822651844.0,    69997945.0 / 29380423.0};

struct Stages
{
  const double *k[7];
  double w[7];
};

// out = x + h sum_j w_j k_j (terms with w_j = 0 skipped)
__global__ void combine_kernel(double *__restrict__ out, const double *__restrict__ x, Stages S, int m, double h,
                               long len)
{
  const long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  double acc = 0.0;
  for (int j = 0; j < m; ++j)
    if (S.w[j] != 0.0) acc += S.w[j] * S.k[j][i];
  out[i] = x[i] + h * acc;
}

// max_i |h sum_j e_j k_j| / (eps_abs + eps_rel (|x_i| + h |k1_i|)) into *err
// (non-negative doubles order as their bit patterns)
__global__ void error_kernel(Stages S, const double *__restrict__ x, double h, double eps_abs, double eps_rel, long len,
                             unsigned long long *__restrict__ err)
{
  double m = 0.0;
  for (long i = (long) blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long) gridDim.x * blockDim.x)
  {
    double e = 0.0;
    for (int j = 0; j < 7; ++j)
      if (S.w[j] != 0.0) e += S.w[j] * S.k[j][i];
    const double r = fabs(h * e) / (eps_abs + eps_rel * (fabs(x[i]) + h * fabs(S.k[0][i])));
    m = fmax(m, r);
  }
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) atomicMax(err, (unsigned long long) __double_as_longlong(m));
}

// y(t_old + theta h) from the step's end points and stages (continuous extension)
__global__ void dense_kernel(double *__restrict__ out, const double *__restrict__ y0, const double *__restrict__ y1,
                             Stages S, double h, double theta, long len)
{
  const long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  double d = 0.0;
  for (int j = 0; j < 7; ++j)
    if (S.w[j] != 0.0) d += S.w[j] * S.k[j][i];
  const double yd = y1[i] - y0[i];
  const double bspl = h * S.k[0][i] - yd;
  const double r4 = yd - h * S.k[6][i] - bspl;
  const double r5 = h * d;
  const double t1 = 1.0 - theta;
  out[i] = y0[i] + theta * (yd + t1 * (bspl + theta * (r4 + t1 * r5)));
}

int blocks(long len)
{
  return (int) std::min<long>((len + 255) / 256, 1L << 30);
}

}  // namespace
}  // namespace spss

using namespace spss;

extern "C" int spss_integrate_dopri5(spss_ctx *ctx, double t0, double t1, double dt_out, double eps_abs,
                                     double eps_rel, spss_observer_fn observer, void *user, long *steps_out)
{
  if (!ctx || !(dt_out > 0.0) || !(t1 >= t0) || !(eps_abs > 0.0) || !(eps_rel >= 0.0)) return SPSS_ERR_INVALID_ARGUMENT;
  if (ctx->p.precision != SPSS_PRECISION_F64 || !ctx->systems.empty()) return SPSS_ERR_NOT_SUPPORTED;
  const long len = (long) ctx->p.n * ctx->s;
  const double *state_ptr = nullptr;
  SPSS_TRY(f64_state_ptr(ctx, &state_ptr));
  double *x = const_cast<double *>(state_ptr);  // the context's state, advanced in place
  DeviceArray<double> buf;
  // k1..k7, zeros (k_prev of the right-hand side), stage state, new state, dense output
  SPSS_TRY(buf.reserve((size_t) len * 11));
  double *k[7];
  for (int j = 0; j < 7; ++j) k[j] = buf.ptr + (size_t) j * len;
  double *zeros = buf.ptr + 7 * (size_t) len, *stage = buf.ptr + 8 * (size_t) len;
  double *xnew = buf.ptr + 9 * (size_t) len, *xout = buf.ptr + 10 * (size_t) len;
  DeviceArray<unsigned long long> err_d;
  SPSS_TRY(err_d.reserve(1));
  std::vector<double> host;
  cudaStream_t st = ctx->stream;
  SPSS_CUDA_TRY(cudaMemsetAsync(buf.ptr, 0, sizeof(double) * (size_t) len * 11, st));
  auto rhs = [&](const double *y, double *out, double h) -> int {
    return f64_evaluate(ctx, ctx->p.variant, y, zeros, out, 0.0, h);
  };
  auto observe = [&](const double *d_y, double t) -> int {
    if (!observer) return 0;
    host.resize((size_t) len);
    if (cudaMemcpyAsync(host.data(), d_y, sizeof(double) * len, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
    {
      cudaGetLastError();
      return SPSS_ERR_CUDA;
    }
    return observer(host.data(), len, t, user) ? 1 : 0;
  };
  double h = dt_out, t = t0;
  long steps = 0;
  int rc = SPSS_OK;
  int stop = observe(x, t0);
  if (stop < 0) return stop;
  long out_index = 1;
  const long n_out = (long) std::floor((t1 - t0) / dt_out + 1e-9);
  SPSS_TRY(rhs(x, k[0], h));  // first same as last: k1 of every later step is the previous k7
  while (!stop && out_index <= n_out)
  {
    // one attempted step of size h from t
    for (int s = 1; s < 7; ++s)
    {
      Stages S{};
      for (int j = 0; j < s; ++j)
      {
        S.k[j] = k[j];
        S.w[j] = kA[s][j];
      }
      combine_kernel<<<blocks(len), 256, 0, st>>>(s == 6 ? xnew : stage, x, S, s, h, len);
      ++ctx->launches;
      SPSS_TRY(check_launch("dopri5 combine_kernel"));
      SPSS_TRY(rhs(s == 6 ? xnew : stage, k[s], kC[s] * h));
    }
    Stages E{};
    for (int j = 0; j < 7; ++j)
    {
      E.k[j] = k[j];
      E.w[j] = kE[j];
    }
    SPSS_CUDA_TRY(cudaMemsetAsync(err_d.ptr, 0, sizeof(unsigned long long), st));
    error_kernel<<<std::min(blocks(len), 4 * 152), 256, 0, st>>>(E, x, h, eps_abs, eps_rel, len, err_d.ptr);
    ++ctx->launches;
    SPSS_TRY(check_launch("dopri5 error_kernel"));
    unsigned long long bits = 0;
    SPSS_CUDA_TRY(cudaMemcpyAsync(&bits, err_d.ptr, sizeof(bits), cudaMemcpyDeviceToHost, st));
    SPSS_CUDA_TRY(cudaStreamSynchronize(st));
    double err;
    std::memcpy(&err, &bits, sizeof(err));
    if (!std::isfinite(err)) return SPSS_ERR_NONFINITE;
    if (err > 1.0)
    {
      h *= std::max(0.9 * std::pow(err, -1.0 / 3.0), 0.2);
      if (!(h > 1e-14 * std::max(1.0, std::fabs(t)))) return SPSS_ERR_NONFINITE;  // step size underflow
      continue;
    }
    // accepted: observer times inside (t, t + h] from the continuous extension
    ++steps;
    const double t_new = t + h;
    Stages Dd{};
    for (int j = 0; j < 7; ++j)
    {
      Dd.k[j] = k[j];
      Dd.w[j] = kD[j];
    }
    while (!stop && out_index <= n_out && t0 + out_index * dt_out <= t_new * (1.0 + 1e-15))
    {
      const double to = t0 + out_index * dt_out;
      const double theta = (to - t) / h;
      dense_kernel<<<blocks(len), 256, 0, st>>>(xout, x, xnew, Dd, h, theta, len);
      ++ctx->launches;
      SPSS_TRY(check_launch("dopri5 dense_kernel"));
      stop = observe(xout, to);
      if (stop < 0) return stop;
      ++out_index;
    }
    if (out_index > n_out)
    {
      // the integration ends at the last observer time: the state there
      const double te = t0 + n_out * dt_out;
      if (n_out > 0 && te < t_new)
      {
        dense_kernel<<<blocks(len), 256, 0, st>>>(xout, x, xnew, Dd, h, (te - t) / h, len);
        ++ctx->launches;
        SPSS_TRY(check_launch("dopri5 dense_kernel"));
        SPSS_CUDA_TRY(cudaMemcpyAsync(x, xout, sizeof(double) * len, cudaMemcpyDeviceToDevice, st));
      } else
      {
        SPSS_CUDA_TRY(cudaMemcpyAsync(x, xnew, sizeof(double) * len, cudaMemcpyDeviceToDevice, st));
      }
      break;
    }
    SPSS_CUDA_TRY(cudaMemcpyAsync(x, xnew, sizeof(double) * len, cudaMemcpyDeviceToDevice, st));
    std::swap(k[0], k[6]);  // first same as last
    t = t_new;
    if (err < 0.5) h *= 0.9 * std::pow(std::max(err, std::pow(5.0, -5.0)), -1.0 / 5.0);
  }
  SPSS_CUDA_TRY(cudaStreamSynchronize(st));
  if (steps_out) *steps_out = steps;
  return rc;
}
