// Drop-in C++ classes with the reference's names and signatures, backed by
// libspss_gpu.so (include/spss_gpu.h).  A program written against the
// reference's ParticleSystem / Stepper / Observer classes compiles against
// this header instead of DynamicalSystems/, Steppers/, Observers/,
// BoundaryConfiguration/ and Parallelization/ and runs the hot path on the
// GPU.  Errors the reference would only assert on throw spss::Error.
//
// Reference interfaces mirrored (file:line in the reference tree):
//   ParticleSystemFirstOrder        DynamicalSystems/ParticleSystemFirstOrder.hpp:12-71
//   ParticleSystemFirstOrderPtr     DynamicalSystems/ParticleSystemFirstOrderPtr.hpp:12-114
//   ParticleSystemSecondOrder       DynamicalSystems/ParticleSystemSecondOrder.hpp:12-106
//   ParticleSystemSecondOrderPtr    DynamicalSystems/ParticleSystemSecondOrderPtr.hpp:12-116
//   RungeKutta4Stepper[Ptr]         Steppers/RungeKutta4Stepper.hpp:15-42, RungeKutta4StepperPtr.hpp:15-35
//   StochasticEulerStepper[Ptr]     Steppers/StochasticEulerStepper.hpp:14-60, StochasticEulerStepperPtr.hpp:19-115
//   StochasticRungeKuttaStepperPtr  Steppers/StochasticRungeKuttaStepperPtr.hpp:21-85
//   PeriodicBoundaryConditions      BoundaryConfiguration/PeriodicBoundaryConditions.hpp:12-48
//   Thread, ThreadSharedMemory      Parallelization/Thread.hpp:12-41, ThreadSharedMemory.hpp:15-53
//   AveragingObserver[Ptr]          Observers/AveragingObserver.hpp:12-35, AveragingObserverPtr.hpp:14-37
//   BinaryObserverFirstOrder[Ptr]   Observers/BinaryObserverFirstOrder.hpp:18-50, BinaryObserverFirstOrderPtr.hpp:18-51
//   BinaryObserverSecondOrder[Ptr]  Observers/BinaryObserverSecondOrder.hpp:16-55, BinaryObserverSecondOrderPtr.hpp:16-57
//
// State residency.  DoStep runs on the GPU and writes the stepped state back
// into the caller's host array; the GPU keeps a copy.  The library remembers,
// per particle system, which host array that copy mirrors (the array most
// recently passed to its DoStep).  PeriodicBoundaryConditions wraps such an
// array on the host as the reference does and wraps the GPU copy with it, and
// the observers read the GPU copy of such an array (GPU order-parameter
// reduction, frames converted on the GPU) instead of looping over the host
// array.  A program that changes a stepped array on the host by other means
// before an observer reads it calls spss::HostStateChanged(array) first; the
// observers then read the host array.
#ifndef SPSS_DROPIN_HPP
#define SPSS_DROPIN_HPP

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <mutex>
#include <numeric>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../spss_gpu.h"

typedef double Real;
typedef float RealOutput;

namespace spss
{

class Error : public std::runtime_error
{
 public:
  Error(int code, const char *what)
      : std::runtime_error(std::string(what) + ": " + spss_error_string(code)), code_(code)
  {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc, const char *what)
{
  if (rc != SPSS_OK) throw Error(rc, what);
}

// Arithmetic of the particle systems constructed from now on:
// SPSS_PRECISION_F64 (the reference's FP64 arithmetic, default) or
// SPSS_PRECISION_F32 (GB300 fast path: stochastic steppers only).
inline int &default_precision()
{
  static int p = SPSS_PRECISION_F64;
  return p;
}

inline unsigned long long &default_seed()
{
  static unsigned long long s = 0;
  return s;
}

// Folder the reference-named observers write into (the reference compiles a
// machine-specific folder into each observer).  Default: the environment
// variable SPSS_OUTPUT_FOLDER, else the working directory; include the
// trailing '/'.
inline std::string &output_folder()
{
  static std::string folder = [] {
    const char *env = std::getenv("SPSS_OUTPUT_FOLDER");
    return std::string(env ? env : "");
  }();
  return folder;
}

// The observers print the reference's "value at t = ... integrated in ...s"
// line on every saved frame; false silences it.
inline bool &observer_progress_lines()
{
  static bool on = true;
  return on;
}

namespace detail
{

// Host arrays mirrored on the GPU: array -> context whose device state is a
// copy of it (set by DoStep; a context mirrors one array at a time).
struct Resident
{
  const void *host;
  spss_ctx *ctx;
};

inline std::mutex &resident_mutex()
{
  static std::mutex m;
  return m;
}

inline std::vector<Resident> &residents()
{
  static std::vector<Resident> r;
  return r;
}

inline void set_resident(const void *host, spss_ctx *ctx)
{
  std::lock_guard<std::mutex> lock(resident_mutex());
  auto &r = residents();
  r.erase(std::remove_if(r.begin(), r.end(), [&](const Resident &e) { return e.host == host || e.ctx == ctx; }),
          r.end());
  r.push_back({host, ctx});
}

inline void drop_resident_host(const void *host)
{
  std::lock_guard<std::mutex> lock(resident_mutex());
  auto &r = residents();
  r.erase(std::remove_if(r.begin(), r.end(), [&](const Resident &e) { return e.host == host; }), r.end());
}

inline void drop_resident_ctx(spss_ctx *ctx)
{
  std::lock_guard<std::mutex> lock(resident_mutex());
  auto &r = residents();
  r.erase(std::remove_if(r.begin(), r.end(), [&](const Resident &e) { return e.ctx == ctx; }), r.end());
}

inline spss_ctx *resident(const void *host)
{
  std::lock_guard<std::mutex> lock(resident_mutex());
  for (const Resident &e : residents())
    if (e.host == host) return e.ctx;
  return nullptr;
}

// Called with a context just before a drop-in particle system destroys it.
struct ContextListener
{
  int id;
  std::function<void(spss_ctx *)> fn;
};

inline std::vector<ContextListener> &context_listeners()
{
  static std::vector<ContextListener> l;
  return l;
}

inline int add_context_listener(std::function<void(spss_ctx *)> fn)
{
  std::lock_guard<std::mutex> lock(resident_mutex());
  static int next = 0;
  context_listeners().push_back({++next, std::move(fn)});
  return next;
}

inline void remove_context_listener(int id)
{
  std::lock_guard<std::mutex> lock(resident_mutex());
  auto &l = context_listeners();
  l.erase(std::remove_if(l.begin(), l.end(), [&](const ContextListener &e) { return e.id == id; }), l.end());
}

inline void notify_context_destroyed(spss_ctx *ctx)
{
  std::vector<ContextListener> copy;
  {
    std::lock_guard<std::mutex> lock(resident_mutex());
    copy = context_listeners();
  }
  for (auto &e : copy) e.fn(ctx);
}

}  // namespace detail

// The program changed `state` on the host after the last DoStep on it: the
// GPU copy no longer mirrors it, and the observers read the host array until
// the next DoStep.
inline void HostStateChanged(const Real *state) { detail::drop_resident_host(state); }

}  // namespace spss

// ------------------------------------------------------------------ Thread

class Thread
{
 public:
  Thread(int, char **, int number_of_particles, int number_of_state_variables)
      : n_(number_of_particles), s_(number_of_state_variables), loop_indices_(number_of_particles)
  {
    std::iota(loop_indices_.begin(), loop_indices_.end(), 0);
  }
  virtual ~Thread() = default;
  int GetRank() { return 0; }
  int GetNumberOfMpichThreads() { return 1; }
  int GetNumberOfParticlesPerMpichThread() { return n_; }
  const std::vector<int> &GetLoopIndices() const { return loop_indices_; }
  virtual bool IsRoot() const { return true; }
  virtual void SynchronizeVector(std::vector<Real> &) {}
  virtual void SynchronizeVectorThoughBuffer(std::vector<Real> &, std::vector<Real> &) {}
  virtual void BroadcastVector(std::vector<Real> &) {}
  virtual void SynchronizePrelinkedList(std::vector<int> &) const {}

 protected:
  int n_;
  int s_;
  std::vector<int> loop_indices_;
};

// One GPU replaces the shared-memory MPI decomposition: every rank-local call is local.
class ThreadSharedMemory : public Thread
{
 public:
  using Thread::Thread;
  using Thread::BroadcastVector;
  using Thread::SynchronizeVector;
  bool IsSharedRoot() { return true; }
  void SynchronizeVector(Real *const, long) {}
  void BroadcastVector(Real *const, long) {}
};

// ------------------------------------------------------------------ PBC

class PeriodicBoundaryConditions
{
 public:
  PeriodicBoundaryConditions(Thread *thread, int number_of_particles, int number_of_state_variables, Real x_size,
                             Real y_size)
      : thread_(thread), n_(number_of_particles), s_(number_of_state_variables), x_size_(x_size), y_size_(y_size),
        x_rsize_(1.0 / x_size), y_rsize_(1.0 / y_size)
  {}
  void ClassAEffectiveParticleDistance(Real x_i, Real y_i, Real x_j, Real y_j, Real &dx, Real &dy) const
  {
    dx = x_j - x_i;
    dx -= static_cast<int>(dx * 2.0 * x_rsize_) * x_size_;
    dy = y_j - y_i;
    dy -= static_cast<int>(dy * 2.0 * y_rsize_) * y_size_;
  }
  void ClassCEffectiveParticleDistanceUnsigned(Real x_i, Real y_i, Real x_j, Real y_j, Real &dx, Real &dy) const
  {
    dx = std::fabs(x_j - x_i);
    dx -= static_cast<int>(dx * x_rsize_ + 0.5) * x_size_;
    dy = std::fabs(y_j - y_i);
    dy -= static_cast<int>(dy * y_rsize_ + 0.5) * y_size_;
  }
  void ApplyPeriodicBoundaryConditions(Real x, Real y, Real &x_pbc, Real &y_pbc) const
  {
    x_pbc = x - std::floor(x * x_rsize_) * x_size_;
    y_pbc = y - std::floor(y * y_rsize_) * y_size_;
  }
  // PeriodicBoundaryConditions::ApplyPeriodicBoundaryConditions (PeriodicBoundaryConditions.cpp:127-155):
  // the host array as the reference wraps it and, when the array is mirrored
  // on the GPU (the last array a drop-in DoStep stepped), the GPU copy too.
  template<class V>
  void ApplyPeriodicBoundaryConditions(V &system_state)
  {
    for (int i = 0; i < n_; ++i)
    {
      system_state[s_ * i] -= std::floor(system_state[s_ * i] * x_rsize_) * x_size_;
      system_state[s_ * i + 1] -= std::floor(system_state[s_ * i + 1] * y_rsize_) * y_size_;
    }
    WrapMirror(&system_state[0]);
  }
  void ApplyPeriodicBoundaryConditions(Real *const system_state, long)
  {
    for (int i = 0; i < n_; ++i)
    {
      system_state[s_ * i] -= std::floor(system_state[s_ * i] * x_rsize_) * x_size_;
      system_state[s_ * i + 1] -= std::floor(system_state[s_ * i + 1] * y_rsize_) * y_size_;
    }
    WrapMirror(system_state);
  }
  Real GetXSize() const { return x_size_; }
  Real GetYSize() const { return y_size_; }

 private:
  void WrapMirror(const void *host)
  {
    if (spss_ctx *ctx = spss::detail::resident(host)) spss::check(spss_apply_pbc(ctx), "ApplyPeriodicBoundaryConditions");
  }

  Thread *thread_;
  int n_, s_;
  Real x_size_, y_size_, x_rsize_, y_rsize_;
};

// ------------------------------------------------------------------ systems

namespace spss
{

// Shared implementation of the four particle-system classes: one GPU context.
class SystemBase
{
 public:
  SystemBase(int model, int flavor, int n, int s, Real v_0, Real xi, Real xi_r, Real D_r, Real xi_phi, Real D_phi,
             Real sigma, Real rho, Real alpha, Real r_max)
      : n_(n), s_(s), rho_(rho), D_r_(D_r), D_phi_(D_phi), xi_(xi), alpha_(alpha)
  {
    spss_params p{};
    p.model = model;
    p.flavor = flavor;
    p.n = n;
    p.variant = SPSS_VARIANT_DISPATCH;
    p.precision = default_precision();
    p.v0 = v_0;
    p.xi = xi;
    p.xi_r = xi_r;
    p.D_r = D_r;
    p.xi_phi = xi_phi;
    p.D_phi = D_phi;
    p.sigma = sigma;
    p.rho = rho;
    p.alpha = alpha;
    p.r_max = r_max;
    p.seed = default_seed();
    params_ = p;
    check(spss_create(&p, &ctx_), "spss_create");
  }
  SystemBase(const SystemBase &) = delete;
  SystemBase &operator=(const SystemBase &) = delete;
  ~SystemBase()
  {
    if (ctx_)
    {
      detail::notify_context_destroyed(ctx_);
      detail::drop_resident_ctx(ctx_);
      spss_destroy(ctx_);
    }
  }

  // Stepper entry: the context runs DoStep on the caller's host array, whose
  // copy then stays on the GPU for the observers.
  void Step(int stepper, Real *state, Real t, Real dt)
  {
    detail::drop_resident_ctx(ctx_);
    check(spss_step_host(ctx_, stepper, state, (long) n_ * s_, t, dt), "DoStep");
    detail::set_resident(state, ctx_);
    RefreshFlags();
  }
  spss_ctx *context() { return ctx_; }
  // Extension (no reference counterpart): choose the interaction routine the
  // steppers use, e.g. the Verlet list for the second-order model.
  void SetVariant(int variant, Real r_max = 0.0, int nc_verlet = 0)
  {
    spss_params p = params_;
    p.variant = variant;
    if (r_max > 0.0) p.r_max = r_max;
    p.nc_verlet = nc_verlet;
    spss_ctx *c = nullptr;
    check(spss_create(&p, &c), "spss_create");
    detail::notify_context_destroyed(ctx_);
    detail::drop_resident_ctx(ctx_);
    spss_destroy(ctx_);
    ctx_ = c;
    params_ = p;
  }

  bool uses_verlet_list_ = false;

 protected:
  void Eval(int variant, const Real *state, const std::vector<Real> &k_prev, std::vector<Real> &k_next, Real k_coef,
            Real dt)
  {
    check(spss_evaluate_rhs(ctx_, variant, state, k_prev.data(), k_next.data(), k_coef, dt), "EvaluateRhs");
    RefreshFlags();
  }
  void RefreshFlags()
  {
    int uses = 0;
    check(spss_get_verlet_state(ctx_, nullptr, nullptr, &uses), "spss_get_verlet_state");
    uses_verlet_list_ = uses != 0;
  }
  void Noise(int stepper, std::vector<Real> &out)
  {
    unsigned long long step = 0;
    check(spss_get_step_counter(ctx_, &step), "spss_get_step_counter");
    check(spss_noise(ctx_, stepper, step, out.data(), (long) out.size()), "spss_noise");
    check(spss_set_step_counter(ctx_, step + 1), "spss_set_step_counter");
  }

  spss_ctx *ctx_ = nullptr;
  spss_params params_{};
  int n_, s_;
  Real rho_, D_r_, D_phi_, xi_, alpha_;
};

}  // namespace spss

class ParticleSystemFirstOrder : public spss::SystemBase
{
 public:
  ParticleSystemFirstOrder(Thread *, Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi,
                           PeriodicBoundaryConditions &, int number_of_particles, int number_of_state_variables)
      : SystemBase(1, 0, number_of_particles, number_of_state_variables, v_0, xi, 0.0, 0.0, 0.0, D_phi, sigma, rho,
                   alpha, 0.0)
  {}
  void SetNaturalFrequencies(const std::vector<Real> &f)
  {
    spss::check(spss_set_natural_frequencies(ctx_, f.data(), (long) f.size()), "SetNaturalFrequencies");
  }
  void EvaluateRhs(const std::vector<Real> &x, const std::vector<Real> &kp, std::vector<Real> &kn, Real c, Real dt)
  {
    Eval(SPSS_VARIANT_DISPATCH, x.data(), kp, kn, c, dt);
  }
  void operator()(const std::vector<Real> &x, std::vector<Real> &d, const Real dt)
  {
    static const std::vector<Real> zero(x.size(), 0.0);
    EvaluateRhs(x, zero, d, 0.0, dt);
  }
  void EvaluateInteractionsWithGlobalPolarOrderField(const std::vector<Real> &x, const std::vector<Real> &kp,
                                                     std::vector<Real> &kn, Real c, Real dt)
  {
    Eval(SPSS_VARIANT_GLOBAL_FIELD, x.data(), kp, kn, c, dt);
  }
  void EvaluateInteractionsWithAllPairs(const std::vector<Real> &x, const std::vector<Real> &kp,
                                        std::vector<Real> &kn, Real c, Real dt)
  {
    Eval(SPSS_VARIANT_ALL_PAIRS, x.data(), kp, kn, c, dt);
  }
  void EvaluateInteractionsWithLinkedList(const std::vector<Real> &x, const std::vector<Real> &kp,
                                          std::vector<Real> &kn, Real c, Real dt)
  {
    Eval(SPSS_VARIANT_LINKED_LIST, x.data(), kp, kn, c, dt);
  }
  void EvaluateInteractionsWithVerletNeighborList(const std::vector<Real> &x, const std::vector<Real> &kp,
                                                  std::vector<Real> &kn, Real c, Real dt)
  {
    Eval(SPSS_VARIANT_VERLET, x.data(), kp, kn, c, dt);
  }
  void EvaluateInteractionsWithLinkedListAndVerletNeighborList(const std::vector<Real> &x,
                                                               const std::vector<Real> &kp, std::vector<Real> &kn,
                                                               Real c, Real dt)
  {
    Eval(SPSS_VARIANT_LINKED_LIST_VERLET, x.data(), kp, kn, c, dt);
  }
  // ParticleSystemFirstOrder::AddNoise (ParticleSystemFirstOrder.cpp:698-708): sqrt(2 D_phi) N(0,1) into omega.
  void AddNoise(const std::vector<Real> &, std::vector<Real> &derivative, Real)
  {
    std::vector<Real> z((size_t) n_);
    Noise(SPSS_STEPPER_STOCHASTIC_EULER, z);
    const Real intensity_phi = std::sqrt(2.0 * D_phi_);
    for (int i = 0; i < n_; ++i) derivative[s_ * i + 3] = intensity_phi * z[i];
  }
  void CalculateMaxDisplacement(const std::vector<Real> &td)
  {
    spss::check(spss_calculate_max_displacement(ctx_, td.data(), (long) td.size()), "CalculateMaxDisplacement");
  }
  Real rho() const { return rho_; }
  Real D_phi() const { return D_phi_; }
};

class ParticleSystemFirstOrderPtr : public spss::SystemBase
{
 public:
  ParticleSystemFirstOrderPtr(ThreadSharedMemory *, Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi,
                              PeriodicBoundaryConditions &, int number_of_particles, int number_of_state_variables)
      : SystemBase(1, 1, number_of_particles, number_of_state_variables, v_0, xi, 0.0, 0.0, 0.0, D_phi, sigma, rho,
                   alpha, 0.0)
  {}
  void SetNaturalFrequencies(const std::vector<Real> &f)
  {
    spss::check(spss_set_natural_frequencies(ctx_, f.data(), (long) f.size()), "SetNaturalFrequencies");
  }
  void EvaluateRhs(const Real *const x, const std::vector<Real> &kp, std::vector<Real> &kn, Real c, Real dt)
  {
    spss::check(spss_set_higher_order(ctx_, is_higher_order_sde_integration_), "spss_set_higher_order");
    Eval(SPSS_VARIANT_DISPATCH, x, kp, kn, c, dt);
  }
  void EvaluateInteractionsWithAllPairs(const Real *const x, const std::vector<Real> &kp, std::vector<Real> &kn,
                                        Real c, Real dt)
  {
    spss::check(spss_set_higher_order(ctx_, is_higher_order_sde_integration_), "spss_set_higher_order");
    Eval(SPSS_VARIANT_ALL_PAIRS, x, kp, kn, c, dt);
  }
  void EvaluateInteractionsWithLinkedList(const Real *const x, const std::vector<Real> &kp, std::vector<Real> &kn,
                                          Real c, Real dt)
  {
    spss::check(spss_set_higher_order(ctx_, is_higher_order_sde_integration_), "spss_set_higher_order");
    Eval(SPSS_VARIANT_LINKED_LIST, x, kp, kn, c, dt);
  }
  void EvaluateInteractionsWithVerletNeighborList(const Real *const x, const std::vector<Real> &kp,
                                                  std::vector<Real> &kn, Real c, Real dt)
  {
    spss::check(spss_set_higher_order(ctx_, is_higher_order_sde_integration_), "spss_set_higher_order");
    Eval(SPSS_VARIANT_VERLET, x, kp, kn, c, dt);
  }
  void EvaluateInteractionsWithLinkedListAndVerletNeighborList(const Real *const x, const std::vector<Real> &kp,
                                                               std::vector<Real> &kn, Real c, Real dt)
  {
    spss::check(spss_set_higher_order(ctx_, is_higher_order_sde_integration_), "spss_set_higher_order");
    Eval(SPSS_VARIANT_LINKED_LIST_VERLET, x, kp, kn, c, dt);
  }
  void CalculateMaxDisplacement(const std::vector<Real> &td)
  {
    spss::check(spss_calculate_max_displacement(ctx_, td.data(), (long) td.size()), "CalculateMaxDisplacement");
  }
  const std::vector<Real> &GetComplimentaryAlignmentForce()
  {
    caf_.resize((size_t) n_);
    spss::check(spss_get_complementary_force(ctx_, caf_.data(), (long) n_), "GetComplimentaryAlignmentForce");
    return caf_;
  }
  Real xi() const { return xi_; }
  Real rho() const { return rho_; }
  Real D_phi() const { return D_phi_; }
  Real alpha() const { return alpha_; }
  bool is_higher_order_sde_integration_ = false;

 private:
  std::vector<Real> caf_;
};

class ParticleSystemSecondOrder : public spss::SystemBase
{
 public:
  ParticleSystemSecondOrder(Thread *, Real v_0, Real xi_r, Real D_r, Real xi_phi, Real D_phi, Real sigma, Real rho,
                            Real alpha, PeriodicBoundaryConditions &, int number_of_particles,
                            int number_of_state_variables)
      : SystemBase(2, 0, number_of_particles, number_of_state_variables, v_0, 0.0, xi_r, D_r, xi_phi, D_phi, sigma,
                   rho, alpha, 0.0)
  {}
  void EvaluateRhs(std::vector<Real> &x, const std::vector<Real> &kp, std::vector<Real> &kn, Real c, Real dt)
  {
    Eval(SPSS_VARIANT_DISPATCH, x.data(), kp, kn, c, dt);
  }
  void EvaluateInteractionsWithAllPairs(std::vector<Real> &x, const std::vector<Real> &kp, std::vector<Real> &kn,
                                        Real c, Real dt)
  {
    Eval(SPSS_VARIANT_ALL_PAIRS, x.data(), kp, kn, c, dt);
  }
  void EvaluateInteractionsWithLinkedList(std::vector<Real> &x, const std::vector<Real> &kp, std::vector<Real> &kn,
                                          Real c, Real dt)
  {
    Eval(SPSS_VARIANT_LINKED_LIST, x.data(), kp, kn, c, dt);
  }
  // ParticleSystemSecondOrder::AddNoise (ParticleSystemSecondOrder.cpp:439-451): draws (r_x, r_y, phi) per particle.
  void AddNoise(const std::vector<Real> &, std::vector<Real> &derivative, Real)
  {
    std::vector<Real> z((size_t) n_ * 3);
    Noise(SPSS_STEPPER_STOCHASTIC_EULER, z);
    const Real ir = std::sqrt(2.0 * D_r_), ip = std::sqrt(2.0 * D_phi_);
    for (int i = 0; i < n_; ++i)
    {
      derivative[s_ * i + 2] = ir * z[3 * i];
      derivative[s_ * i + 3] = ir * z[3 * i + 1];
      derivative[s_ * i + 5] = ip * z[3 * i + 2];
    }
  }
  Real rho() const { return rho_; }
  Real D_r() const { return D_r_; }
  Real D_phi() const { return D_phi_; }
  bool last_coefficient_ = true;
};

class ParticleSystemSecondOrderPtr : public spss::SystemBase
{
 public:
  ParticleSystemSecondOrderPtr(ThreadSharedMemory *, Real v_0, Real xi_r, Real D_r, Real xi_phi, Real D_phi,
                               Real sigma, Real rho, Real alpha, PeriodicBoundaryConditions &, int number_of_particles,
                               int number_of_state_variables)
      : SystemBase(2, 1, number_of_particles, number_of_state_variables, v_0, 0.0, xi_r, D_r, xi_phi, D_phi, sigma,
                   rho, alpha, 0.0)
  {}
  void EvaluateRhs(const Real *const x, const std::vector<Real> &kp, std::vector<Real> &kn, Real c, Real dt)
  {
    Eval(SPSS_VARIANT_DISPATCH, x, kp, kn, c, dt);
  }
  void EvaluateInteractionsWithAllPairs(const Real *const x, const std::vector<Real> &kp, std::vector<Real> &kn,
                                        Real c, Real dt)
  {
    Eval(SPSS_VARIANT_ALL_PAIRS, x, kp, kn, c, dt);
  }
  void EvaluateInteractionsWithLinkedList(const Real *const x, const std::vector<Real> &kp, std::vector<Real> &kn,
                                          Real c, Real dt)
  {
    Eval(SPSS_VARIANT_LINKED_LIST, x, kp, kn, c, dt);
  }
  // The reference leaves this a stub (ParticleSystemSecondOrderPtr.cpp:393-400); here it is the
  // restated second-order Verlet routine.
  void EvaluateInteractionsWithVerletNeighborList(const Real *const x, const std::vector<Real> &kp,
                                                  std::vector<Real> &kn, Real c, Real dt)
  {
    Eval(SPSS_VARIANT_LINKED_LIST_VERLET, x, kp, kn, c, dt);
  }
  Real rho() const { return rho_; }
  Real D_r() const { return D_r_; }
  Real D_phi() const { return D_phi_; }
  bool last_coefficient_ = true;
};

// ------------------------------------------------------------------ steppers

class RungeKutta4Stepper
{
 public:
  RungeKutta4Stepper(Thread *, int, int) {}
  void DoStep(ParticleSystemFirstOrder &sys, std::vector<Real> &x, Real t, Real dt)
  {
    sys.Step(SPSS_STEPPER_RK4, x.data(), t, dt);
  }
  void DoStep(ParticleSystemSecondOrder &sys, std::vector<Real> &x, Real t, Real dt)
  {
    sys.Step(SPSS_STEPPER_RK4, x.data(), t, dt);
  }
};

class RungeKutta4StepperPtr
{
 public:
  RungeKutta4StepperPtr(ThreadSharedMemory *, int, int) {}
  void DoStep(ParticleSystemFirstOrderPtr &sys, Real *const x, Real t, Real dt) { sys.Step(SPSS_STEPPER_RK4, x, t, dt); }
  void DoStep(ParticleSystemSecondOrderPtr &sys, Real *const x, Real t, Real dt)
  {
    sys.Step(SPSS_STEPPER_RK4, x, t, dt);
  }
};

class StochasticEulerStepper
{
 public:
  StochasticEulerStepper(Thread *, int, int) {}
  void DoStep(ParticleSystemSecondOrder &sys, std::vector<Real> &x, Real t, Real dt)
  {
    sys.Step(SPSS_STEPPER_STOCHASTIC_EULER, x.data(), t, dt);
  }
};

class StochasticEulerStepperPtr
{
 public:
  StochasticEulerStepperPtr(ThreadSharedMemory *, int, int) {}
  void DoStep(ParticleSystemFirstOrderPtr &sys, Real *const x, Real t, Real dt)
  {
    sys.Step(SPSS_STEPPER_STOCHASTIC_EULER, x, t, dt);
  }
  // the reference's second-order branch asserts (StochasticEulerStepperPtr.hpp:97); here it runs
  void DoStep(ParticleSystemSecondOrderPtr &sys, Real *const x, Real t, Real dt)
  {
    sys.Step(SPSS_STEPPER_STOCHASTIC_EULER, x, t, dt);
  }
};

class StochasticRungeKuttaStepperPtr
{
 public:
  StochasticRungeKuttaStepperPtr(ThreadSharedMemory *, int, int) {}
  void DoStep(ParticleSystemFirstOrderPtr &sys, Real *const x, Real t, Real dt)
  {
    sys.is_higher_order_sde_integration_ = true;
    sys.Step(SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA, x, t, dt);
  }
  // second-order strong order 1.5 scheme: no reference counterpart
  void DoStep(ParticleSystemSecondOrderPtr &sys, Real *const x, Real t, Real dt)
  {
    sys.Step(SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA, x, t, dt);
  }
};

// ------------------------------------------------------------------ observers

namespace spss
{
namespace detail
{

constexpr double kTwoPi = 6.283185307179586476925286766559;

// The .bin trajectory file of a binary observer: frames [float t][float s*n]
// (BinaryObserverFirstOrder.cpp:119-120).  Frames of a GPU-mirrored state are
// converted on the GPU (spss_frame_async) into one of two page-locked
// buffers and written by a background thread while the next steps run;
// frames of a host array are converted and written on the calling thread.
// Frames reach the file in call order.
class FrameFile
{
 public:
  FrameFile(const std::string &path, long len) : len_(len)
  {
    std::remove(path.c_str());
    file_ = std::fopen(path.c_str(), "ab");
    if (!file_) throw Error(SPSS_ERR_INVALID_ARGUMENT, ("cannot open " + path).c_str());
  }
  FrameFile(const FrameFile &) = delete;
  FrameFile &operator=(const FrameFile &) = delete;
  ~FrameFile()
  {
    Flush();
    for (float *b : buf_)
      if (b) spss_pinned_free(b);
    if (file_) std::fclose(file_);
  }
  void Flush()
  {
    for (auto &w : writer_)
      if (w.joinable()) w.join();
  }
  // The frame of the state `ctx` holds (SPSS_FRAME_RAW or SPSS_FRAME_WRAPPED).
  void WriteDevice(spss_ctx *ctx, int mode, float t)
  {
    const int b = next_;
    if (writer_[b].joinable()) writer_[b].join();  // this buffer's previous frame is on disk
    if (!buf_[b]) check(spss_pinned_alloc(sizeof(float) * (size_t) len_, (void **) &buf_[b]), "spss_pinned_alloc");
    check(spss_frame_async(ctx, mode, buf_[b], len_), "spss_frame_async");
    check(spss_synchronize(ctx), "spss_synchronize");
    if (writer_[1 - b].joinable()) writer_[1 - b].join();  // the previous frame goes first
    FILE *f = file_;
    float *frame = buf_[b];
    const long len = len_;
    writer_[b] = std::thread([f, t, frame, len]() {
      std::fwrite(&t, sizeof(float), 1, f);
      std::fwrite(frame, sizeof(float), (size_t) len, f);
    });
    next_ = 1 - b;
  }
  void WriteHost(const float *frame, float t)
  {
    Flush();
    std::fwrite(&t, sizeof(float), 1, file_);
    std::fwrite(frame, sizeof(float), (size_t) len_, file_);
  }

 private:
  FILE *file_ = nullptr;
  long len_;
  int next_ = 0;
  float *buf_[2] = {nullptr, nullptr};
  std::thread writer_[2];
};

// |<e^{i phi}>| and its argument.  A GPU-mirrored state is reduced on the GPU
// (spss_order_parameters), a host array here; both accumulate in FP64 (the
// reference accumulates complex<float>, BinaryObserverSecondOrder.cpp:181-188).
inline void order_parameter(const Real *x, int n, int s, double &abs_r, double &arg_r)
{
  if (spss_ctx *ctx = resident(x))
  {
    double r[4];
    check(spss_order_parameters(ctx, r), "SaveSummaryStatistics");
    abs_r = r[0];
    arg_r = r[1];
    return;
  }
  const int ip = s == 4 ? 2 : 4;
  double re = 0.0, im = 0.0;
  for (int i = 0; i < n; ++i)
  {
    re += std::cos(x[(long) s * i + ip]);
    im += std::sin(x[(long) s * i + ip]);
  }
  re /= n;
  im /= n;
  abs_r = std::sqrt(re * re + im * im);
  arg_r = std::atan2(im, re);
}

}  // namespace detail
}  // namespace spss

namespace spss
{
namespace detail
{

// Shared body of the four reference binary observers: the two output files,
// the save cadence (output_time_threshold_) and the progress line.
class BinaryObserverBase
{
 protected:
  BinaryObserverBase(PeriodicBoundaryConditions &pbc, int n, int s, int threshold, bool wrapped,
                     const std::string &simulation_file_name, const std::string &summary_file_name)
      : pbc_(pbc), n_(n), s_(s), threshold_(threshold), wrapped_(wrapped),
        frames_(simulation_file_name, (long) n * s), timer_(std::chrono::system_clock::now())
  {
    std::remove(summary_file_name.c_str());
    summary_.open(summary_file_name, std::ios::out | std::ios::app);
    if (!summary_.is_open()) throw Error(SPSS_ERR_INVALID_ARGUMENT, ("cannot open " + summary_file_name).c_str());
  }

  void ProgressLine(Real t)
  {
    const std::chrono::duration<Real> elapsed = std::chrono::system_clock::now() - timer_;
    if (observer_progress_lines())
      std::cout << "value at t = " << t << " integrated in " << elapsed.count() << "s" << std::endl;
    timer_ = std::chrono::system_clock::now();
  }

  // One frame: BinaryObserverFirstOrder::SaveSystemState (BinaryObserverFirstOrder.cpp:110-120: float
  // state, positions wrapped into the box and the phase into [0, 2 pi), each wrap evaluated in double on
  // the float and rounded back) or BinaryObserverSecondOrder::SaveSystemState
  // (BinaryObserverSecondOrder.cpp:111-116: the float state).
  void Frame(const Real *x, Real t)
  {
    const float tf = (float) t;
    spss_ctx *ctx = resident(x);
    const bool unit_box = pbc_.GetXSize() == 1.0 && pbc_.GetYSize() == 1.0;
    if (ctx && (unit_box || !wrapped_))
    {
      frames_.WriteDevice(ctx, wrapped_ ? SPSS_FRAME_WRAPPED : SPSS_FRAME_RAW, tf);
      return;
    }
    host_frame_.assign(x, x + (size_t) n_ * s_);
    if (wrapped_)
    {
      pbc_.ApplyPeriodicBoundaryConditions(host_frame_);
      for (int i = 0; i < n_; ++i)
        host_frame_[(size_t) s_ * i + 2] -= std::floor(host_frame_[(size_t) s_ * i + 2] / kTwoPi) * kTwoPi;
    }
    frames_.WriteHost(host_frame_.data(), tf);
  }

  // One summary line "t \t |R| \t arg R" (BinaryObserverFirstOrder.cpp:125-142).
  void Summary(const Real *x, Real t)
  {
    double abs_r, arg_r;
    order_parameter(x, n_, s_, abs_r, arg_r);
    summary_ << (float) t << '\t' << (float) abs_r << '\t' << (float) arg_r << std::endl;
  }

  PeriodicBoundaryConditions &pbc_;
  int n_, s_;
  int threshold_;
  bool wrapped_;
  FrameFile frames_;
  std::ofstream summary_;
  std::vector<float> host_frame_;
  std::chrono::time_point<std::chrono::system_clock> timer_;
  int counter_[2] = {0, 0};
};

}  // namespace detail
}  // namespace spss

// BinaryObserverFirstOrder (Observers/BinaryObserverFirstOrder.hpp:18-50, .cpp:18-147): every 100th call
// writes a wrapped float frame and a summary line, to files named after the parameters.
class BinaryObserverFirstOrder : public spss::detail::BinaryObserverBase
{
 public:
  BinaryObserverFirstOrder(Thread *, Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi,
                           PeriodicBoundaryConditions &pbc_config, int number_of_particles,
                           int number_of_state_variables, Real, int trial)
      : BinaryObserverBase(pbc_config, number_of_particles, number_of_state_variables, 100, true,
                           Name(v_0, xi, sigma, rho, alpha, D_phi, number_of_particles, trial, true),
                           Name(v_0, xi, sigma, rho, alpha, D_phi, number_of_particles, trial, false))
  {}
  void SaveSystemState(const std::vector<Real> &system_state, Real t)
  {
    if (!(counter_[0] % threshold_))
    {
      ProgressLine(t);
      Frame(system_state.data(), t);
    }
    ++counter_[0];
  }
  void SaveSummaryStatistics(const std::vector<Real> &system_state, Real t)
  {
    if (!(counter_[1] % threshold_)) Summary(system_state.data(), t);
    ++counter_[1];
  }
  void operator()(const std::vector<Real> &system_state, Real t)
  {
    SaveSystemState(system_state, t);
    SaveSummaryStatistics(system_state, t);
  }
  // File names of BinaryObserverFirstOrder.cpp:50-76 (the trajectory's alpha onwards at 10 digits).
  static std::string Name(Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi, int n, int trial,
                          bool trajectory)
  {
    std::ostringstream b;
    b << spss::output_folder() << "v0_" << v_0 << "_xi_" << xi << "_sigma_" << sigma << "_rho_" << rho << "_alpha_";
    if (trajectory) b << std::setprecision(10);
    b << alpha << "_Dphi_" << D_phi << "_N_" << n << "_" << 0 << "_" << trial << (trajectory ? ".bin" : ".txt");
    return b.str();
  }
};

// BinaryObserverFirstOrderPtr (Observers/BinaryObserverFirstOrderPtr.hpp:18-51, .cpp:20-147): as the serial
// observer; the progress line comes on every SaveSystemState call.
class BinaryObserverFirstOrderPtr : public spss::detail::BinaryObserverBase
{
 public:
  BinaryObserverFirstOrderPtr(ThreadSharedMemory *, Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi,
                              PeriodicBoundaryConditions &pbc_config, int number_of_particles,
                              int number_of_state_variables, Real, int trial)
      : BinaryObserverBase(pbc_config, number_of_particles, number_of_state_variables, 100, true,
                           Name(v_0, xi, sigma, rho, alpha, D_phi, number_of_particles, trial, ".bin"),
                           Name(v_0, xi, sigma, rho, alpha, D_phi, number_of_particles, trial, ".txt"))
  {}
  void SaveSystemState(Real *const system_state, long, Real t)
  {
    ProgressLine(t);
    if (!(counter_[0] % threshold_)) Frame(system_state, t);
    ++counter_[0];
  }
  void SaveSummaryStatistics(const Real *const system_state, long, Real t)
  {
    if (!(counter_[1] % threshold_)) Summary(system_state, t);
    ++counter_[1];
  }
  // File names of BinaryObserverFirstOrderPtr.cpp:52-70.
  static std::string Name(Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi, int n, int trial,
                          const char *ext)
  {
    std::ostringstream b;
    b << spss::output_folder() << "v0_" << v_0 << "_xi_" << xi << "_sigma_" << sigma << "_rho_" << rho << "_alpha_"
      << alpha << "_Dphi_" << D_phi << "_N_" << n << "_" << 0 << "_" << trial << ext;
    return b.str();
  }
};

// Trajectory and summary file names of BinaryObserverSecondOrder.cpp:50-80 and
// BinaryObserverSecondOrderPtr.cpp:51-69.
inline std::string SecondOrderObserverName(Real v_0, Real xi_r, Real D_r, Real xi_phi, Real D_phi, Real sigma,
                                           Real rho, Real alpha, int n, int trial, bool trajectory)
{
  std::ostringstream b;
  b << spss::output_folder() << (trajectory ? "" : "summary_statistics_") << "v0_" << v_0 << "_xir_" << xi_r
    << "_Dr_" << D_r << "_xiphi_" << xi_phi << "_Dphi_" << D_phi << "_sigma_" << sigma << "_rho_" << rho
    << "_alpha_" << alpha << "_N_" << n << "_" << 0 << "_" << trial << (trajectory ? ".bin" : ".txt");
  return b.str();
}

// BinaryObserverSecondOrder (Observers/BinaryObserverSecondOrder.hpp:16-55, .cpp:14-138): every 10th call
// writes the float state and a summary line.
class BinaryObserverSecondOrder : public spss::detail::BinaryObserverBase
{
 public:
  BinaryObserverSecondOrder(Thread *, Real v_0, Real xi_r, Real D_r, Real xi_phi, Real D_phi, Real sigma, Real rho,
                            Real alpha, PeriodicBoundaryConditions &pbc_config, int number_of_particles,
                            int number_of_state_variables, Real, int trial)
      : BinaryObserverBase(pbc_config, number_of_particles, number_of_state_variables, 10, false,
                           SecondOrderObserverName(v_0, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
                                                   number_of_particles, trial, true),
                           SecondOrderObserverName(v_0, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
                                                   number_of_particles, trial, false))
  {}
  void SaveSystemState(std::vector<Real> &system_state, Real t)
  {
    if (!(counter_[0] % threshold_))
    {
      ProgressLine(t);
      Frame(system_state.data(), t);
    }
    ++counter_[0];
  }
  void SaveSummaryStatistics(std::vector<Real> &system_state, Real t)
  {
    if (!(counter_[1] % threshold_)) Summary(system_state.data(), t);
    ++counter_[1];
  }
};

// BinaryObserverSecondOrderPtr (Observers/BinaryObserverSecondOrderPtr.hpp:16-57, .cpp:15-196).
class BinaryObserverSecondOrderPtr : public spss::detail::BinaryObserverBase
{
 public:
  BinaryObserverSecondOrderPtr(ThreadSharedMemory *, Real v_0, Real xi_r, Real D_r, Real xi_phi, Real D_phi,
                               Real sigma, Real rho, Real alpha, PeriodicBoundaryConditions &pbc_config,
                               int number_of_particles, int number_of_state_variables, Real, int trial)
      : BinaryObserverBase(pbc_config, number_of_particles, number_of_state_variables, 10, false,
                           SecondOrderObserverName(v_0, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
                                                   number_of_particles, trial, true),
                           SecondOrderObserverName(v_0, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
                                                   number_of_particles, trial, false))
  {}
  void SaveSystemState(Real *const system_state, long, Real t)
  {
    if (!(counter_[0] % threshold_))
    {
      ProgressLine(t);
      Frame(system_state, t);
    }
    ++counter_[0];
  }
  void SaveSummaryStatistics(const Real *const system_state, long, Real t)
  {
    if (!(counter_[1] % threshold_)) Summary(system_state, t);
    ++counter_[1];
  }
};

namespace spss
{
namespace detail
{

// Shared body of AveragingObserver[Ptr]: the running sum of the state
// (AveragingObserver.cpp:29-37).  Calls on a GPU-mirrored state add the GPU
// copy on the GPU (spss_average_accumulate, FP64) into the accumulator of the
// system that stepped it; other calls add the host array here.  One averaging
// observer at a time uses a system's accumulator (another one sums on the
// host); a system destroyed before the average is saved hands its sums over
// first.
class AveragingObserverBase
{
 protected:
  AveragingObserverBase(int n, int s) : n_(n), s_(s), sum_((size_t) n * s, 0.0)
  {
    listener_ = add_context_listener([this](spss_ctx *ctx) {
      if (ctx == dev_) Fold();
    });
  }
  ~AveragingObserverBase()
  {
    remove_context_listener(listener_);
    if (dev_) Release(dev_);
  }
  AveragingObserverBase(const AveragingObserverBase &) = delete;
  AveragingObserverBase &operator=(const AveragingObserverBase &) = delete;

  void Accumulate(const Real *x)
  {
    spss_ctx *ctx = resident(x);
    if (ctx && ctx != dev_)
    {
      Fold();
      if (Claim(ctx)) Attach(ctx);
    }
    if (ctx && ctx == dev_)
    {
      check(spss_average_accumulate(ctx), "AveragingObserver");
    } else
    {
      for (size_t q = 0; q < sum_.size(); ++q) sum_[q] += x[q];
    }
    ++count_;
  }

  // AveragingObserver::SaveAveragedSystemState (AveragingObserver.cpp:39-68): the averaged omega
  // (component 3) of every particle as float, to a file named after the parameters.
  void Save(Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi, int trial)
  {
    Fold();
    std::ostringstream b;
    b << output_folder() << "averaged_angular_velocities_v0_" << v_0 << "_xi_" << xi << "_sigma_" << sigma
      << "_rho_" << rho << "_alpha_" << std::setprecision(10) << alpha << "_Dphi_" << D_phi << "_N_" << n_ << "_"
      << trial << ".bin";
    std::ofstream file(b.str(), std::ios::out | std::ios::trunc | std::ios::binary);
    if (!file.is_open()) throw Error(SPSS_ERR_INVALID_ARGUMENT, ("cannot open " + b.str()).c_str());
    std::vector<RealOutput> w((size_t) n_);
    for (int i = 0; i < n_; ++i) w[i] = sum_[(size_t) s_ * i + 3] / count_;
    file.write((const char *) w.data(), n_ * sizeof(RealOutput));
  }

 public:
  // Sum of the states accumulated so far (host and GPU calls) and their number.
  const std::vector<Real> &AccumulatedSystemState()
  {
    Fold();
    return sum_;
  }
  int NumberOfAccumulatedSteps() const { return count_; }

 private:
  static std::vector<spss_ctx *> &claimed()
  {
    static std::vector<spss_ctx *> c;
    return c;
  }
  static bool Claim(spss_ctx *ctx)
  {
    std::lock_guard<std::mutex> lock(resident_mutex());
    auto &c = claimed();
    if (std::find(c.begin(), c.end(), ctx) != c.end()) return false;
    c.push_back(ctx);
    return true;
  }
  static void Release(spss_ctx *ctx)
  {
    std::lock_guard<std::mutex> lock(resident_mutex());
    auto &c = claimed();
    c.erase(std::remove(c.begin(), c.end(), ctx), c.end());
  }
  // The GPU accumulator's current sums and count.
  void DeviceSums(spss_ctx *ctx, std::vector<Real> &sums, int &count)
  {
    sums.resize(sum_.size());
    check(spss_average_get(ctx, sums.data(), (long) sums.size(), &count), "AveragingObserver");
    for (Real &v : sums) v *= count;
  }
  void Attach(spss_ctx *ctx)
  {
    dev_ = ctx;
    DeviceSums(ctx, base_, base_count_);
  }
  // Move what this observer added on the GPU since Attach into the host sums.
  void Fold()
  {
    if (!dev_) return;
    std::vector<Real> now;
    int count = 0;
    DeviceSums(dev_, now, count);
    if (count > base_count_)
      for (size_t q = 0; q < sum_.size(); ++q) sum_[q] += now[q] - base_[q];
    Release(dev_);
    dev_ = nullptr;
  }

  int n_, s_;
  std::vector<Real> sum_, base_;
  int count_ = 0, base_count_ = 0;
  spss_ctx *dev_ = nullptr;
  int listener_ = 0;
};

}  // namespace detail
}  // namespace spss

// AveragingObserver (Observers/AveragingObserver.hpp:12-35, .cpp:13-68).
class AveragingObserver : public spss::detail::AveragingObserverBase
{
 public:
  AveragingObserver(int number_of_particles, int number_of_state_variables)
      : AveragingObserverBase(number_of_particles, number_of_state_variables)
  {}
  void operator()(const std::vector<Real> &system_state, Real) { Accumulate(system_state.data()); }
  void SaveAveragedSystemState(Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi, int trial)
  {
    Save(v_0, xi, sigma, rho, alpha, D_phi, trial);
  }
};

// AveragingObserverPtr (Observers/AveragingObserverPtr.hpp:14-37, .cpp:13-78).
class AveragingObserverPtr : public spss::detail::AveragingObserverBase
{
 public:
  AveragingObserverPtr(ThreadSharedMemory *, int number_of_particles, int number_of_state_variables)
      : AveragingObserverBase(number_of_particles, number_of_state_variables)
  {}
  void operator()(Real *const system_state, long, Real) { Accumulate(system_state); }
  void SaveAveragedSystemState(Real v_0, Real xi, Real sigma, Real rho, Real alpha, Real D_phi, int trial)
  {
    Save(v_0, xi, sigma, rho, alpha, D_phi, trial);
  }
};

namespace spss
{

// Binary observer on the GPU state of one system, at a cadence of the
// caller's choice and with file names of the caller's choice: frames in the
// reference's .bin format computed on the GPU, written by a background thread
// while the next steps run; optional summary lines (t, |R|, arg R).
// `wrapped` follows BinaryObserverFirstOrder (positions and phases wrapped),
// otherwise BinaryObserverSecondOrder (the state as it is).  No counterpart in
// the reference beyond the file formats.
class TrajectoryWriter
{
 public:
  TrajectoryWriter(spss::SystemBase &system, int number_of_particles, int number_of_state_variables,
                   const std::string &trajectory_file, const std::string &summary_file, int every, bool wrapped)
      : ctx_(system.context()), every_(every), mode_(wrapped ? SPSS_FRAME_WRAPPED : SPSS_FRAME_RAW),
        frames_(trajectory_file, (long) number_of_particles * number_of_state_variables)
  {
    if (!summary_file.empty()) summ_ = std::fopen(summary_file.c_str(), "w");
  }
  TrajectoryWriter(const TrajectoryWriter &) = delete;
  TrajectoryWriter &operator=(const TrajectoryWriter &) = delete;
  ~TrajectoryWriter()
  {
    frames_.Flush();
    if (summ_) std::fclose(summ_);
  }
  void operator()(Real t)
  {
    if (!(counter_++ % every_))
    {
      frames_.WriteDevice(ctx_, mode_, (float) t);
      if (summ_)
      {
        double r[4];
        spss::check(spss_order_parameters(ctx_, r), "spss_order_parameters");
        std::fprintf(summ_, "%g\t%g\t%g\n", (float) t, (float) r[0], (float) r[1]);
      }
    }
  }

 private:
  spss_ctx *ctx_;
  int every_, mode_;
  int counter_ = 0;
  detail::FrameFile frames_;
  FILE *summ_ = nullptr;
};

// The last frame of a .bin trajectory file as the initial state
// (SimulationEngineFirstOrder::InitializeSystemStateFromPreviousSolution,
// SimulationEngineFirstOrder.cpp:69-93); returns the frame's time.
inline Real ReadLastFrame(const std::string &file, int number_of_particles, int number_of_state_variables, Real *state)
{
  FILE *f = std::fopen(file.c_str(), "rb");
  if (!f) throw std::runtime_error("ReadLastFrame: cannot open " + file);
  const long per = 1L + (long) number_of_particles * number_of_state_variables;
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  const long frames = size / (per * (long) sizeof(float));
  if (frames < 1)
  {
    std::fclose(f);
    throw std::runtime_error("ReadLastFrame: no whole frame in " + file);
  }
  std::fseek(f, (frames - 1) * per * (long) sizeof(float), SEEK_SET);
  std::vector<float> raw((size_t) per);
  const size_t got = std::fread(raw.data(), sizeof(float), (size_t) per, f);
  std::fclose(f);
  if (got != (size_t) per) throw std::runtime_error("ReadLastFrame: short read from " + file);
  std::copy(raw.begin() + 1, raw.end(), state);
  return (Real) raw[0];
}

}  // namespace spss

#endif
