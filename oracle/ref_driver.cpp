// Driver that runs the reference's own hot-path classes, compiled unmodified
// from their source tree, on one input and dumps every intermediate the
// golden fixtures need.  Test infrastructure only: the product never links it.
//
// Usage: spss_ref <config.txt>
//   config.txt holds "key value" lines (see ReadConfig).  Arrays are raw
//   little-endian float64 files named in the config.  Outputs are written to
//   <out>_<name>.bin (float64 or int32) and <out>_meta.txt.
//
// One configuration per process: the reference keeps function-local static
// buffers sized at their first call (e.g. ParticleSystemFirstOrder.cpp:175,
// StochasticRungeKuttaStepperPtr.hpp:42), so a second configuration in the
// same process would reuse wrongly sized buffers.

#include <algorithm>
#include <cassert>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>
#include <mpi.h>

// Private members (cell lists, Verlet lists, trigger state) are read for the
// bit-exact fixtures.  Standard headers are already included above.
#define private public
#include "Definitions.hpp"
#include "BoundaryConfiguration/PeriodicBoundaryConditions.hpp"
#include "Parallelization/Thread.hpp"
#include "Parallelization/ThreadSharedMemory.hpp"
#include "DynamicalSystems/ParticleSystemFirstOrder.hpp"
#include "DynamicalSystems/ParticleSystemFirstOrderPtr.hpp"
#include "DynamicalSystems/ParticleSystemSecondOrder.hpp"
#include "DynamicalSystems/ParticleSystemSecondOrderPtr.hpp"
#include "Steppers/RungeKutta4Stepper.hpp"
#include "Steppers/RungeKutta4StepperPtr.hpp"
#include "Steppers/StochasticEulerStepper.hpp"
#include "Steppers/StochasticEulerStepperPtr.hpp"
#include "Steppers/StochasticRungeKuttaStepperPtr.hpp"
#undef private

std::mt19937 mersenne_twister_generator(0u);

namespace spss_replay
{
static std::vector<double> buffer;
static size_t position = 0;
double next()
{
  if (position >= buffer.size())
  {
    std::fprintf(stderr, "spss_ref: noise replay buffer exhausted after %zu draws\n", position);
    std::exit(3);
  }
  return buffer[position++];
}
}

static std::map<std::string, std::string> ReadConfig(const char *path)
{
  std::map<std::string, std::string> cfg;
  std::ifstream f(path);
  if (!f)
  {
    std::fprintf(stderr, "spss_ref: cannot open %s\n", path);
    std::exit(2);
  }
  std::string line;
  while (std::getline(f, line))
  {
    std::istringstream ss(line);
    std::string key, value;
    if (ss >> key >> value) cfg[key] = value;
  }
  return cfg;
}

static std::vector<double> ReadDoubles(const std::string &path, size_t expected)
{
  std::vector<double> v(expected, 0.0);
  if (path.empty() || path == "-") return v;
  std::ifstream f(path, std::ios::binary);
  if (!f)
  {
    std::fprintf(stderr, "spss_ref: cannot open %s\n", path.c_str());
    std::exit(2);
  }
  f.read(reinterpret_cast<char *>(v.data()), expected * sizeof(double));
  return v;
}

static std::vector<double> ReadAllDoubles(const std::string &path)
{
  std::vector<double> v;
  if (path.empty() || path == "-") return v;
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) return v;
  std::streamsize bytes = f.tellg();
  f.seekg(0);
  v.resize(bytes / sizeof(double));
  f.read(reinterpret_cast<char *>(v.data()), bytes);
  return v;
}

template<class T>
static void Write(const std::string &path, const T *data, size_t count)
{
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  f.write(reinterpret_cast<const char *>(data), count * sizeof(T));
}

// CSR dump of a vector<vector<int>>: [rows+1 offsets][entries].
static void WriteCsr(const std::string &path, const std::vector<std::vector<int>> &lists)
{
  std::vector<int> out;
  out.reserve(lists.size() + 1);
  int offset = 0;
  out.push_back(0);
  for (const auto &l : lists)
  {
    offset += (int) l.size();
    out.push_back(offset);
  }
  for (const auto &l : lists) out.insert(out.end(), l.begin(), l.end());
  Write(path, out.data(), out.size());
}

struct Config
{
  int model = 1;          // 1 first order, 2 second order
  std::string flavor;     // "serial" or "ptr"
  std::string mode;       // "rhs" or "step"
  int variant = 0;        // 0 dispatch, 1 all-pairs, 2 linked list, 3 Verlet, 4 LL+Verlet, 5 global field
  std::string stepper;    // rk4, rk4_direct, se, srk
  int n = 0;
  int nsteps = 1;
  int higher_order = 0;
  double v0 = 0, xi = 0, xi_r = 0, D_r = 0, xi_phi = 0, D_phi = 0, sigma = 0, rho = 0, alpha = 0;
  double k_coef = 0, dt = 0, t0 = 0;
  std::string state, kprev, knext, noise, freqs, out;
};

static Config Parse(const std::map<std::string, std::string> &m)
{
  Config c;
  auto get = [&](const char *k, const std::string &def) {
    auto it = m.find(k);
    return it == m.end() ? def : it->second;
  };
  c.model = std::stoi(get("model", "1"));
  c.flavor = get("flavor", "serial");
  c.mode = get("mode", "rhs");
  c.variant = std::stoi(get("variant", "0"));
  c.stepper = get("stepper", "rk4");
  c.n = std::stoi(get("n", "0"));
  c.nsteps = std::stoi(get("nsteps", "1"));
  c.higher_order = std::stoi(get("higher_order", "0"));
  c.v0 = std::stod(get("v0", "0"));
  c.xi = std::stod(get("xi", "0"));
  c.xi_r = std::stod(get("xi_r", "0"));
  c.D_r = std::stod(get("D_r", "0"));
  c.xi_phi = std::stod(get("xi_phi", "0"));
  c.D_phi = std::stod(get("D_phi", "0"));
  c.sigma = std::stod(get("sigma", "0"));
  c.rho = std::stod(get("rho", "0"));
  c.alpha = std::stod(get("alpha", "0"));
  c.k_coef = std::stod(get("k_coef", "0"));
  c.dt = std::stod(get("dt", "0.01"));
  c.t0 = std::stod(get("t0", "0"));
  c.state = get("state", "");
  c.kprev = get("kprev", "");
  c.knext = get("knext", "");
  c.noise = get("noise", "");
  c.freqs = get("freqs", "");
  c.out = get("out", "out");
  return c;
}

static void WriteMeta(const Config &c, double acc, int flag, int uses_verlet, size_t draws)
{
  std::ofstream f(c.out + "_meta.txt", std::ios::trunc);
  f.precision(17);
  f << "accumulated_displacement " << acc << "\n";
  f << "should_update_lists " << flag << "\n";
  f << "uses_verlet_list " << uses_verlet << "\n";
  f << "noise_draws " << draws << "\n";
}

// ---------------------------------------------------------------- first order
template<class System, class State>
static void EvalFirst(System &sys, int variant, State state, const std::vector<Real> &kp, std::vector<Real> &kn,
                      Real k_coef, Real dt)
{
  switch (variant)
  {
    case 0: sys.EvaluateRhs(state, kp, kn, k_coef, dt); break;
    case 1: sys.EvaluateInteractionsWithAllPairs(state, kp, kn, k_coef, dt); break;
    case 2: sys.EvaluateInteractionsWithLinkedList(state, kp, kn, k_coef, dt); break;
    case 3: sys.EvaluateInteractionsWithVerletNeighborList(state, kp, kn, k_coef, dt); break;
    case 4: sys.EvaluateInteractionsWithLinkedListAndVerletNeighborList(state, kp, kn, k_coef, dt); break;
    case 5: sys.EvaluateInteractionsWithGlobalPolarOrderField(state, kp, kn, k_coef, dt); break;
    default: std::fprintf(stderr, "bad variant\n"); std::exit(2);
  }
}

template<class System, class State>
static void EvalSecond(System &sys, int variant, State state, const std::vector<Real> &kp, std::vector<Real> &kn,
                       Real k_coef, Real dt)
{
  switch (variant)
  {
    case 0: sys.EvaluateRhs(state, kp, kn, k_coef, dt); break;
    case 1: sys.EvaluateInteractionsWithAllPairs(state, kp, kn, k_coef, dt); break;
    case 2: sys.EvaluateInteractionsWithLinkedList(state, kp, kn, k_coef, dt); break;
    default: std::fprintf(stderr, "bad variant\n"); std::exit(2);
  }
}

// RK4 with a directly chosen interaction routine.  The combine is that of
// RungeKutta4Stepper::DoStep (Steppers/RungeKutta4Stepper.cpp:29-64); it lets
// a fixture pin e.g. all-pairs RK4 at an interaction radius for which the
// reference's own rho-dispatch would pick another routine.
template<class Eval>
static void Rk4Direct(Eval eval, std::vector<Real> &x, std::vector<Real> &k1, std::vector<Real> &k2,
                      std::vector<Real> &k3, std::vector<Real> &k4, Real dt)
{
  eval(k1, k1, 0.0);
  eval(k1, k2, 0.5);
  eval(k2, k3, 0.5);
  eval(k3, k4, 1.0);
  for (size_t q = 0; q < x.size(); ++q)
  {
    x[q] += (k1[q] + 2.0 * k2[q] + 2.0 * k3[q] + k4[q]) * dt / 6.0;
  }
}

static void DumpFirst(const Config &c, ParticleSystemFirstOrder &sys)
{
  Write(c.out + "_pll.bin", sys.pre_linked_list_.data(), sys.pre_linked_list_.size());
  WriteCsr(c.out + "_cells.bin", sys.linked_list_);
  WriteCsr(c.out + "_verlet.bin", sys.verlet_list_);
}

static void DumpFirstPtr(const Config &c, ParticleSystemFirstOrderPtr &sys)
{
  Write(c.out + "_pll.bin", sys.pre_linked_list_, (size_t) c.n);
  WriteCsr(c.out + "_cells.bin", sys.linked_list_);
  WriteCsr(c.out + "_verlet.bin", sys.verlet_list_);
  const std::vector<Real> &caf = sys.GetComplimentaryAlignmentForce();
  Write(c.out + "_caf.bin", caf.data(), caf.size());
}

static void DumpSecond(const Config &c, ParticleSystemSecondOrder &sys)
{
  Write(c.out + "_pll.bin", sys.pre_linked_list_.data(), sys.pre_linked_list_.size());
  WriteCsr(c.out + "_cells.bin", sys.linked_list_);
}

static void DumpSecondPtr(const Config &c, ParticleSystemSecondOrderPtr &sys)
{
  Write(c.out + "_pll.bin", sys.pre_linked_list_, (size_t) c.n);
  WriteCsr(c.out + "_cells.bin", sys.linked_list_);
}

int main(int argc, char **argv)
{
  if (argc < 2)
  {
    std::fprintf(stderr, "usage: spss_ref <config.txt>\n");
    return 2;
  }
  Config c = Parse(ReadConfig(argv[1]));
  const int s = (c.model == 1) ? 4 : 6;
  const size_t len = (size_t) c.n * s;
  std::vector<Real> state = ReadDoubles(c.state, len);
  std::vector<Real> kprev = ReadDoubles(c.kprev, len);
  std::vector<Real> knext = ReadDoubles(c.knext, len);
  spss_replay::buffer = ReadAllDoubles(c.noise);
  spss_replay::position = 0;

  Thread thread(argc, argv, c.n, s);
  ThreadSharedMemory *shm = nullptr;
  if (c.flavor == "ptr") shm = new ThreadSharedMemory(argc, argv, c.n, s);
  PeriodicBoundaryConditions pbc(c.flavor == "ptr" ? (Thread *) shm : &thread, c.n, s, 1.0, 1.0);

  double acc = 0.0;
  int flag = 0, uses_verlet = 0;
  if (c.model == 1 && c.flavor == "serial")
  {
    ParticleSystemFirstOrder sys(&thread, c.v0, c.xi, c.sigma, c.rho, c.alpha, c.D_phi, pbc, c.n, s);
    if (!c.freqs.empty()) sys.SetNaturalFrequencies(ReadDoubles(c.freqs, c.n));
    if (c.mode == "rhs")
    {
      EvalFirst(sys, c.variant, state, kprev, knext, c.k_coef, c.dt);
    } else if (c.stepper == "rk4")
    {
      RungeKutta4Stepper stepper(&thread, c.n, s);
      Real t = c.t0;
      for (int k = 0; k < c.nsteps; ++k)
      {
        t += c.dt;
        stepper.DoStep(sys, state, t, c.dt);
      }
    } else if (c.stepper == "rk4_direct")
    {
      std::vector<Real> k1(len, 0.0), k2(len, 0.0), k3(len, 0.0), k4(len, 0.0);
      for (int k = 0; k < c.nsteps; ++k)
      {
        Rk4Direct([&](const std::vector<Real> &kp, std::vector<Real> &kn, Real kc) {
          EvalFirst(sys, c.variant, state, kp, kn, kc, c.dt);
        }, state, k1, k2, k3, k4, c.dt);
      }
    } else
    {
      std::fprintf(stderr, "stepper %s not available for the serial first-order class\n", c.stepper.c_str());
      return 2;
    }
    DumpFirst(c, sys);
    acc = sys.accumulated_displacement_;
    flag = sys.should_update_lists_;
    uses_verlet = sys.uses_verlet_list_;
  } else if (c.model == 1)
  {
    ParticleSystemFirstOrderPtr sys(shm, c.v0, c.xi, c.sigma, c.rho, c.alpha, c.D_phi, pbc, c.n, s);
    if (!c.freqs.empty()) sys.SetNaturalFrequencies(ReadDoubles(c.freqs, c.n));
    sys.is_higher_order_sde_integration_ = (c.higher_order != 0);
    Real *raw = new Real[len];
    std::copy(state.begin(), state.end(), raw);
    if (c.mode == "rhs")
    {
      EvalFirst(sys, c.variant, (const Real *) raw, kprev, knext, c.k_coef, c.dt);
    } else
    {
      Real t = c.t0;
      if (c.stepper == "rk4")
      {
        RungeKutta4StepperPtr stepper(shm, c.n, s);
        for (int k = 0; k < c.nsteps; ++k)
        {
          t += c.dt;
          stepper.DoStep(sys, raw, t, c.dt);
        }
      } else if (c.stepper == "se")
      {
        StochasticEulerStepperPtr stepper(shm, c.n, s);
        for (int k = 0; k < c.nsteps; ++k)
        {
          t += c.dt;
          stepper.DoStep(sys, raw, t, c.dt);
        }
      } else if (c.stepper == "srk")
      {
        StochasticRungeKuttaStepperPtr stepper(shm, c.n, s);
        for (int k = 0; k < c.nsteps; ++k)
        {
          t += c.dt;
          stepper.DoStep(sys, raw, t, c.dt);
        }
      } else
      {
        std::fprintf(stderr, "unknown stepper %s\n", c.stepper.c_str());
        return 2;
      }
    }
    std::copy(raw, raw + len, state.begin());
    delete[] raw;
    DumpFirstPtr(c, sys);
    acc = sys.accumulated_displacement_;
    flag = sys.should_update_lists_;
    uses_verlet = sys.uses_verlet_list_;
  } else if (c.flavor == "serial")
  {
    ParticleSystemSecondOrder sys(&thread, c.v0, c.xi_r, c.D_r, c.xi_phi, c.D_phi, c.sigma, c.rho, c.alpha, pbc, c.n, s);
    if (c.mode == "rhs")
    {
      EvalSecond(sys, c.variant, state, kprev, knext, c.k_coef, c.dt);
    } else
    {
      Real t = c.t0;
      if (c.stepper == "rk4")
      {
        RungeKutta4Stepper stepper(&thread, c.n, s);
        for (int k = 0; k < c.nsteps; ++k)
        {
          t += c.dt;
          stepper.DoStep(sys, state, t, c.dt);
        }
      } else if (c.stepper == "se")
      {
        StochasticEulerStepper stepper(&thread, c.n, s);
        for (int k = 0; k < c.nsteps; ++k)
        {
          t += c.dt;
          stepper.DoStep(sys, state, t, c.dt);
        }
      } else if (c.stepper == "rk4_direct")
      {
        std::vector<Real> k1(len, 0.0), k2(len, 0.0), k3(len, 0.0), k4(len, 0.0);
        for (int k = 0; k < c.nsteps; ++k)
        {
          Rk4Direct([&](const std::vector<Real> &kp, std::vector<Real> &kn, Real kc) {
            EvalSecond(sys, c.variant, state, kp, kn, kc, c.dt);
          }, state, k1, k2, k3, k4, c.dt);
        }
      } else
      {
        std::fprintf(stderr, "stepper %s not available for the serial second-order class\n", c.stepper.c_str());
        return 2;
      }
    }
    DumpSecond(c, sys);
    acc = sys.accumulated_displacement_;
    flag = sys.should_update_lists_;
  } else
  {
    ParticleSystemSecondOrderPtr sys(shm, c.v0, c.xi_r, c.D_r, c.xi_phi, c.D_phi, c.sigma, c.rho, c.alpha, pbc, c.n, s);
    Real *raw = new Real[len];
    std::copy(state.begin(), state.end(), raw);
    if (c.mode == "rhs")
    {
      EvalSecond(sys, c.variant, (const Real *) raw, kprev, knext, c.k_coef, c.dt);
    } else if (c.stepper == "rk4")
    {
      RungeKutta4StepperPtr stepper(shm, c.n, s);
      Real t = c.t0;
      for (int k = 0; k < c.nsteps; ++k)
      {
        t += c.dt;
        stepper.DoStep(sys, raw, t, c.dt);
      }
    } else
    {
      std::fprintf(stderr, "stepper %s not available for the MPI second-order class\n", c.stepper.c_str());
      return 2;
    }
    std::copy(raw, raw + len, state.begin());
    delete[] raw;
    DumpSecondPtr(c, sys);
    acc = sys.accumulated_displacement_;
    flag = sys.should_update_lists_;
  }

  if (c.mode == "rhs")
  {
    Write(c.out + "_knext.bin", knext.data(), knext.size());
  } else
  {
    Write(c.out + "_state.bin", state.data(), state.size());
  }
  WriteMeta(c, acc, flag, uses_verlet, spss_replay::position);
  delete shm;
  return 0;
}
