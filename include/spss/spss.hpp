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
//   AveragingObserver               Observers/AveragingObserver.hpp:12-35
//   BinaryObserver{First,Second}Order (SaveSummaryStatistics, SaveSystemState)
#ifndef SPSS_DROPIN_HPP
#define SPSS_DROPIN_HPP

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <numeric>
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
  template<class V>
  void ApplyPeriodicBoundaryConditions(V &system_state)
  {
    for (int i = 0; i < n_; ++i)
    {
      system_state[s_ * i] -= std::floor(system_state[s_ * i] * x_rsize_) * x_size_;
      system_state[s_ * i + 1] -= std::floor(system_state[s_ * i + 1] * y_rsize_) * y_size_;
    }
  }
  void ApplyPeriodicBoundaryConditions(Real *const system_state, long)
  {
    for (int i = 0; i < n_; ++i)
    {
      system_state[s_ * i] -= std::floor(system_state[s_ * i] * x_rsize_) * x_size_;
      system_state[s_ * i + 1] -= std::floor(system_state[s_ * i + 1] * y_rsize_) * y_size_;
    }
  }
  Real GetXSize() const { return x_size_; }
  Real GetYSize() const { return y_size_; }

 private:
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
    if (ctx_) spss_destroy(ctx_);
  }

  // Stepper entry: the context runs DoStep on the caller's host array.
  void Step(int stepper, Real *state, Real t, Real dt)
  {
    check(spss_step_host(ctx_, stepper, state, (long) n_ * s_, t, dt), "DoStep");
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

// AveragingObserver (Observers/AveragingObserver.cpp:29-69): running sum of the state.
class AveragingObserver
{
 public:
  AveragingObserver(int number_of_particles, int number_of_state_variables)
      : n_(number_of_particles), s_(number_of_state_variables), acc_((size_t) number_of_particles * number_of_state_variables, 0.0)
  {}
  void operator()(const std::vector<Real> &x, Real)
  {
    for (size_t q = 0; q < acc_.size(); ++q) acc_[q] += x[q];
    ++count_;
  }
  // averaged omega (index 3) as float, as SaveAveragedSystemState writes it (AveragingObserver.cpp:291-297)
  std::vector<RealOutput> AveragedAngularVelocities() const
  {
    std::vector<RealOutput> out((size_t) n_);
    for (int i = 0; i < n_; ++i) out[i] = acc_[(size_t) s_ * i + 3] / count_;
    return out;
  }
  void SaveAveragedSystemState(const std::string &file_name) const
  {
    std::vector<RealOutput> w = AveragedAngularVelocities();
    FILE *f = std::fopen(file_name.c_str(), "wb");
    if (!f) throw spss::Error(SPSS_ERR_INVALID_ARGUMENT, "SaveAveragedSystemState");
    std::fwrite(w.data(), sizeof(RealOutput), w.size(), f);
    std::fclose(f);
  }
  int count() const { return count_; }

 private:
  int n_, s_;
  std::vector<Real> acc_;
  int count_ = 0;
};

// Order parameter of BinaryObserver*::SaveSummaryStatistics
// (BinaryObserverFirstOrder.cpp:125-142, BinaryObserverSecondOrder.cpp:121-138),
// accumulated in complex<float> as the reference does; phase index 2 (first
// order) or 4 (second order).  Writes "t \t |R| \t arg R" lines and, on the
// observer's cadence, float frames [t][state] of SaveSystemState.
class BinaryObserver
{
 public:
  BinaryObserver(int number_of_particles, int number_of_state_variables, const std::string &trajectory_file,
                 const std::string &summary_file, int every = 10)
      : n_(number_of_particles), s_(number_of_state_variables), every_(every)
  {
    if (!trajectory_file.empty()) traj_ = std::fopen(trajectory_file.c_str(), "wb");
    if (!summary_file.empty()) summ_ = std::fopen(summary_file.c_str(), "w");
  }
  ~BinaryObserver()
  {
    if (traj_) std::fclose(traj_);
    if (summ_) std::fclose(summ_);
  }
  std::complex<float> OrderParameter(const Real *x) const
  {
    const int ip = s_ == 4 ? 2 : 4;
    std::complex<float> r(0.0f, 0.0f);
    for (int i = 0; i < n_; ++i) r += std::complex<float>((float) std::cos(x[s_ * i + ip]), (float) std::sin(x[s_ * i + ip]));
    return r / (float) n_;
  }
  void SaveSystemState(const Real *x, Real t)
  {
    if (traj_ && !(counter_[0] % every_))
    {
      float tf = (float) t;
      std::vector<float> frame(x, x + (size_t) n_ * s_);
      std::fwrite(&tf, sizeof(float), 1, traj_);
      std::fwrite(frame.data(), sizeof(float), frame.size(), traj_);
    }
    ++counter_[0];
  }
  void SaveSummaryStatistics(const Real *x, Real t)
  {
    if (summ_ && !(counter_[1] % every_))
    {
      std::complex<float> r = OrderParameter(x);
      std::fprintf(summ_, "%g\t%g\t%g\n", (float) t, std::abs(r), std::arg(r));
    }
    ++counter_[1];
  }

 private:
  int n_, s_, every_;
  int counter_[2] = {0, 0};
  FILE *traj_ = nullptr;
  FILE *summ_ = nullptr;
};

namespace spss
{

// Binary observer on the GPU state of a system: frames in the reference's
// .bin format ([float t][float s*n]) computed on the GPU (spss_frame_async)
// into page-locked buffers and written by a background thread while the next
// steps run; optional summary lines (t, |R|, arg R).  `wrapped` follows
// BinaryObserverFirstOrder (positions and phases wrapped), otherwise
// BinaryObserverSecondOrder (the state as it is).  No counterpart in the
// reference beyond the file formats.
class TrajectoryWriter
{
 public:
  TrajectoryWriter(spss::SystemBase &system, int number_of_particles, int number_of_state_variables,
                   const std::string &trajectory_file, const std::string &summary_file, int every, bool wrapped)
      : ctx_(system.context()), len_((long) number_of_particles * number_of_state_variables), every_(every),
        mode_(wrapped ? SPSS_FRAME_WRAPPED : SPSS_FRAME_RAW)
  {
    traj_ = std::fopen(trajectory_file.c_str(), "wb");
    if (!traj_) throw std::runtime_error("TrajectoryWriter: cannot open " + trajectory_file);
    if (!summary_file.empty()) summ_ = std::fopen(summary_file.c_str(), "w");
    for (int b = 0; b < 2; ++b)
      spss::check(spss_pinned_alloc(sizeof(float) * (size_t) len_, (void **) &buf_[b]), "spss_pinned_alloc");
  }
  TrajectoryWriter(const TrajectoryWriter &) = delete;
  TrajectoryWriter &operator=(const TrajectoryWriter &) = delete;
  ~TrajectoryWriter()
  {
    for (auto &w : writer_)
      if (w.joinable()) w.join();
    for (float *b : buf_)
      if (b) spss_pinned_free(b);
    if (traj_) std::fclose(traj_);
    if (summ_) std::fclose(summ_);
  }
  void operator()(Real t)
  {
    if (!(counter_++ % every_))
    {
      const int b = next_;
      if (writer_[b].joinable()) writer_[b].join();  // this buffer's previous frame is on disk
      spss::check(spss_frame_async(ctx_, mode_, buf_[b], len_), "spss_frame_async");
      if (summ_)
      {
        double r[4];
        spss::check(spss_order_parameters(ctx_, r), "spss_order_parameters");  // synchronises the stream
        std::fprintf(summ_, "%g\t%g\t%g\n", (float) t, (float) r[0], (float) r[1]);
      } else
      {
        spss::check(spss_synchronize(ctx_), "spss_synchronize");
      }
      // frames reach the file in order: the previous frame's writer finishes first
      if (writer_[1 - b].joinable()) writer_[1 - b].join();
      const float tf = (float) t;
      float *frame = buf_[b];
      FILE *f = traj_;
      const long len = len_;
      writer_[b] = std::thread([f, tf, frame, len]() {
        std::fwrite(&tf, sizeof(float), 1, f);
        std::fwrite(frame, sizeof(float), (size_t) len, f);
      });
      next_ = 1 - b;
    }
  }

 private:
  spss_ctx *ctx_;
  long len_;
  int every_, mode_;
  int counter_ = 0, next_ = 0;
  float *buf_[2] = {nullptr, nullptr};
  std::thread writer_[2];
  FILE *traj_ = nullptr;
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
