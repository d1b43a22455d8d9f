// The reference's engine loops, written against the drop-in classes and run
// on the GB300 path (SPSS_PRECISION_F32):
//   A  SimulationEngineSecondOrder::RunSimulation (ControlEngines/SimulationEngineSecondOrder.cpp:118-143):
//      ParticleSystemSecondOrder, StochasticEulerStepper, PBC after every step, BinaryObserverSecondOrder;
//   B  SimulationEngineSecondOrderPtr::RunSimulation (SimulationEngineSecondOrderPtr.cpp:83-99):
//      ParticleSystemSecondOrderPtr on the restated Verlet list, StochasticRungeKuttaStepperPtr,
//      BinaryObserverSecondOrderPtr;
//   C  SimulationEngineFirstOrderPtr::RunSimulation (SimulationEngineFirstOrderPtr.cpp:122-161):
//      ParticleSystemFirstOrderPtr, StochasticRungeKuttaStepperPtr, BinaryObserverFirstOrderPtr, then the
//      averaging pass on a copy of the state with AveragingObserverPtr.
// Before every DoStep the program records the normals the step will draw
// (spss_noise), so tests/test_gpu_engine_loops.py can replay them in the
// oracle.  Built and run by that test.
//
// usage: engine_loops <dir>   reads <dir>/{a,b,c}_init.bin, writes into <dir>/ the observers' files,
//                              {a,b,c}_final.bin, {a,b,c}_noise.bin, c_avg_final.bin, c_avg_noise.bin, steps.txt
#include <cstdio>
#include <string>
#include <vector>

#include "spss/spss.hpp"

static std::vector<Real> read_all(const std::string &path, size_t n)
{
  std::vector<Real> v(n);
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f || std::fread(v.data(), sizeof(Real), n, f) != n) throw std::runtime_error("read " + path);
  std::fclose(f);
  return v;
}

static void write_all(const std::string &path, const Real *v, size_t n)
{
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("write " + path);
  std::fwrite(v, sizeof(Real), n, f);
  std::fclose(f);
}

// The normals the next DoStep of `system` draws, appended to `out`.
static void record_noise(spss::SystemBase &system, int stepper, long count, std::vector<Real> &out)
{
  unsigned long long step = 0;
  spss::check(spss_get_step_counter(system.context(), &step), "spss_get_step_counter");
  std::vector<Real> z((size_t) count);
  spss::check(spss_noise(system.context(), stepper, step, z.data(), count), "spss_noise");
  out.insert(out.end(), z.begin(), z.end());
}

int main(int argc, char **argv)
{
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  spss::output_folder() = dir + "/";
  spss::observer_progress_lines() = false;
  spss::default_precision() = SPSS_PRECISION_F32;
  spss::default_seed() = 17;
  FILE *steps_file = std::fopen((dir + "/steps.txt").c_str(), "w");
  try
  {
    const int n = 4096;
    const Real t_0 = 0.0, t_1 = 0.25, dt = 0.005;
    {
      // A: second order, stochastic Euler, linked list by the reference's dispatch (rho <= 0.25)
      const int s = 6;
      const Real v_0 = 0.01, xi_r = 1.0, D_r = 1e-4, xi_phi = 1.0, D_phi = 0.1, sigma = 1.0, rho = 0.03,
                 alpha = 0.2;
      const int trial = 0;
      Thread thread(argc, argv, n, s);
      PeriodicBoundaryConditions pbc_config(&thread, n, s, 1.0, 1.0);
      std::vector<Real> system_state = read_all(dir + "/a_init.bin", (size_t) n * s);
      std::vector<Real> noise;
      StochasticEulerStepper stepper(&thread, n, s);
      ParticleSystemSecondOrder particle_system(&thread, v_0, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
                                                pbc_config, n, s);
      BinaryObserverSecondOrder binary_observer(&thread, v_0, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
                                                pbc_config, n, s, dt, trial);
      Real t = t_0;
      int steps = 0;
      binary_observer.SaveSystemState(system_state, t);
      while (t <= t_1)
      {
        t += dt;
        record_noise(particle_system, SPSS_STEPPER_STOCHASTIC_EULER, 3L * n, noise);
        stepper.DoStep(particle_system, system_state, t, dt);
        pbc_config.ApplyPeriodicBoundaryConditions(system_state);
        thread.SynchronizeVector(system_state);
        if (thread.IsRoot())
        {
          binary_observer.SaveSystemState(system_state, t);
          binary_observer.SaveSummaryStatistics(system_state, t);
        }
        ++steps;
      }
      write_all(dir + "/a_final.bin", system_state.data(), system_state.size());
      write_all(dir + "/a_noise.bin", noise.data(), noise.size());
      std::fprintf(steps_file, "%d\n", steps);
    }
    {
      // B: second order, the restated Verlet list (skin 0.3 rho), strong order 1.5 SRK
      const int s = 6;
      const long size = (long) n * s;
      const Real v_0 = 0.01, xi_r = 1.0, D_r = 1e-4, xi_phi = 1.0, D_phi = 0.1, sigma = 1.0, rho = 0.03,
                 alpha = 0.2;
      const int trial = 1;
      ThreadSharedMemory thread(argc, argv, n, s);
      PeriodicBoundaryConditions pbc_config(&thread, n, s, 1.0, 1.0);
      std::vector<Real> init = read_all(dir + "/b_init.bin", (size_t) size);
      Real *system_state = new Real[size];
      std::copy(init.begin(), init.end(), system_state);
      std::vector<Real> noise;
      StochasticRungeKuttaStepperPtr stepper(&thread, n, s);
      ParticleSystemSecondOrderPtr particle_system(&thread, v_0, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
                                                   pbc_config, n, s);
      particle_system.SetVariant(SPSS_VARIANT_LINKED_LIST_VERLET, 1.3 * rho, (int) (1.0 / (1.3 * rho)));
      BinaryObserverSecondOrderPtr binary_observer(&thread, v_0, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
                                                   pbc_config, n, s, dt, trial);
      Real t = t_0;
      int steps = 0;
      binary_observer.SaveSystemState(system_state, size, t);
      while (t <= t_1)
      {
        t += dt;
        record_noise(particle_system, SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA, 6L * n, noise);
        stepper.DoStep(particle_system, system_state, t, dt);
        pbc_config.ApplyPeriodicBoundaryConditions(system_state, size);
        binary_observer.SaveSystemState(system_state, size, t);
        binary_observer.SaveSummaryStatistics(system_state, size, t);
        ++steps;
      }
      write_all(dir + "/b_final.bin", system_state, (size_t) size);
      write_all(dir + "/b_noise.bin", noise.data(), noise.size());
      std::fprintf(steps_file, "%d\n", steps);
      delete[] system_state;
    }
    {
      // C: first order, linked list + Verlet by the reference's dispatch, SRK with the complementary force,
      // positions never wrapped; then the averaging pass
      const int s = 4;
      const long size = (long) n * s;
      const Real v_0 = 0.01, xi = 0.1, sigma = 1.0, rho = 0.03, alpha = 0.3, D_phi = 0.01;
      const Real t_1_first_order = 0.6;  // 121 steps: frames at the 0th and 100th call
      const int trial = 2;
      ThreadSharedMemory thread(argc, argv, n, s);
      PeriodicBoundaryConditions pbc_config(&thread, n, s, 1.0, 1.0);
      std::vector<Real> init = read_all(dir + "/c_init.bin", (size_t) size);
      Real *system_state = new Real[size];
      std::copy(init.begin(), init.end(), system_state);
      std::vector<Real> noise;
      StochasticRungeKuttaStepperPtr stepper(&thread, n, s);
      ParticleSystemFirstOrderPtr particle_system(&thread, v_0, xi, sigma, rho, alpha, D_phi, pbc_config, n, s);
      BinaryObserverFirstOrderPtr binary_observer(&thread, v_0, xi, sigma, rho, alpha, D_phi, pbc_config, n, s, dt,
                                                  trial);
      Real t = t_0;
      int steps = 0;
      binary_observer.SaveSystemState(system_state, size, t);
      while (t <= t_1_first_order)
      {
        t += dt;
        record_noise(particle_system, SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA, 2L * n, noise);
        stepper.DoStep(particle_system, system_state, t, dt);
        binary_observer.SaveSystemState(system_state, size, t);
        binary_observer.SaveSummaryStatistics(system_state, size, t);
        ++steps;
      }
      write_all(dir + "/c_final.bin", system_state, (size_t) size);
      write_all(dir + "/c_noise.bin", noise.data(), noise.size());
      std::fprintf(steps_file, "%d\n", steps);

      Real *averaging_system_state = new Real[size];
      std::copy(&system_state[0], &system_state[size], &averaging_system_state[0]);
      std::vector<Real> avg_noise;
      AveragingObserverPtr averaging_observer(&thread, n, s);
      t = 0.0;
      int avg_steps = 0;
      while (t <= 0.1)
      {
        t += dt;
        record_noise(particle_system, SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA, 2L * n, avg_noise);
        stepper.DoStep(particle_system, averaging_system_state, t, dt);
        averaging_observer.operator()(averaging_system_state, size, t);
        ++avg_steps;
      }
      averaging_observer.SaveAveragedSystemState(v_0, xi, sigma, rho, alpha, D_phi, trial);
      write_all(dir + "/c_avg_final.bin", averaging_system_state, (size_t) size);
      write_all(dir + "/c_avg_noise.bin", avg_noise.data(), avg_noise.size());
      std::fprintf(steps_file, "%d\n", avg_steps);
      delete[] averaging_system_state;
      delete[] system_state;
    }
  } catch (const std::exception &e)
  {
    std::fprintf(stderr, "engine_loops: %s\n", e.what());
    return 1;
  }
  std::fclose(steps_file);
  std::printf("ok\n");
  return 0;
}
