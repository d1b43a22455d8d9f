// Uses the drop-in classes exactly as the reference's engines use theirs
// (ControlEngines/SimulationEngineSecondOrder.cpp:122-143): construct
// Thread, PeriodicBoundaryConditions, a particle system and a stepper, then
// call DoStep in a loop.  Built and run by tests/test_gpu_dropin.py, which
// checks the written states against the oracle.
//
// usage: dropin_example <dir>   reads <dir>/fo_init.bin, <dir>/so_init.bin
//                                writes fo_final.bin, so_final.bin, so_noise.bin,
//                                fo_traj.bin, fo_summary.txt, fo_restart.bin,
//                                {fo,so}_addnoise.bin, {fo,so}_addnoise_z.bin, so_residency.bin
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

static void write_all(const std::string &path, const std::vector<Real> &v)
{
  FILE *f = std::fopen(path.c_str(), "wb");
  std::fwrite(v.data(), sizeof(Real), v.size(), f);
  std::fclose(f);
}

int main(int argc, char **argv)
{
  if (argc < 2) return 2;
  const std::string dir = argv[1];
  try
  {
    {
      // first order, serial class, RK4, rho = 0.1 -> linked list + Verlet by the reference's dispatch
      const int n = 400, s = 4;
      Thread thread(argc, argv, n, s);
      PeriodicBoundaryConditions pbc(&thread, n, s, 1.0, 1.0);
      ParticleSystemFirstOrder system(&thread, 0.3, 0.1, 1.0, 0.1, 0.2, 0.1, pbc, n, s);
      RungeKutta4Stepper stepper(&thread, n, s);
      std::vector<Real> x = read_all(dir + "/fo_init.bin", (size_t) n * s);
      Real t = 0.0, dt = 0.01;
      {
        // the binary observer every 2 steps, wrapped as the first-order observer
        spss::TrajectoryWriter writer(system, n, s, dir + "/fo_traj.bin", dir + "/fo_summary.txt", 2, true);
        for (int k = 0; k < 10; ++k)
        {
          t += dt;
          stepper.DoStep(system, x, t, dt);
          writer(t);
        }
      }
      write_all(dir + "/fo_final.bin", x);
      // restart from the last frame written
      std::vector<Real> restart((size_t) n * s);
      const Real t_last = spss::ReadLastFrame(dir + "/fo_traj.bin", n, s, restart.data());
      restart.push_back(t_last);
      write_all(dir + "/fo_restart.bin", restart);
      if (!system.uses_verlet_list_) throw std::runtime_error("uses_verlet_list_ not set");
    }
    {
      // second order, serial class, stochastic Euler, linked list; noise of each step recorded
      const int n = 500, s = 6;
      Thread thread(argc, argv, n, s);
      PeriodicBoundaryConditions pbc(&thread, n, s, 1.0, 1.0);
      ParticleSystemSecondOrder system(&thread, 0.5, 1.0, 0.02, 1.0, 0.1, 1.0, 0.07, 0.0, pbc, n, s);
      StochasticEulerStepper stepper(&thread, n, s);
      std::vector<Real> x = read_all(dir + "/so_init.bin", (size_t) n * s);
      std::vector<Real> noise;
      Real t = 0.0, dt = 0.005;
      for (int k = 0; k < 5; ++k)
      {
        std::vector<Real> z((size_t) n * 3);
        spss::check(spss_noise(system.context(), SPSS_STEPPER_STOCHASTIC_EULER, (unsigned long long) k, z.data(),
                               (long) z.size()), "spss_noise");
        noise.insert(noise.end(), z.begin(), z.end());
        t += dt;
        stepper.DoStep(system, x, t, dt);
        pbc.ApplyPeriodicBoundaryConditions(x);
      }
      write_all(dir + "/so_final.bin", x);
      write_all(dir + "/so_noise.bin", noise);

      // AddNoise (ParticleSystemSecondOrder.cpp:439-451) twice into a derivative buffer; the
      // normals of the second call recorded
      std::vector<Real> derivative((size_t) n * s, 7.0), z((size_t) n * 3);
      system.AddNoise(x, derivative, t);
      unsigned long long step = 0;
      spss::check(spss_get_step_counter(system.context(), &step), "spss_get_step_counter");
      spss::check(spss_noise(system.context(), SPSS_STEPPER_STOCHASTIC_EULER, step, z.data(), (long) z.size()),
                  "spss_noise");
      system.AddNoise(x, derivative, t);
      write_all(dir + "/so_addnoise.bin", derivative);
      write_all(dir + "/so_addnoise_z.bin", z);

      // State residency: the observers read the GPU copy of a stepped array
      // until the program declares a host change.  All phases set to 0 on the
      // host: the order parameter is still the GPU copy's, then 1 after
      // spss::HostStateChanged.
      std::vector<Real> residency(4);
      spss::detail::order_parameter(x.data(), n, s, residency[0], residency[1]);
      for (int i = 0; i < n; ++i) x[(size_t) s * i + 4] = 0.0;
      spss::detail::order_parameter(x.data(), n, s, residency[2], residency[3]);
      spss::HostStateChanged(x.data());
      double host_r = 0.0, host_arg = 1.0;
      spss::detail::order_parameter(x.data(), n, s, host_r, host_arg);
      residency.push_back(host_r);
      residency.push_back(host_arg);
      write_all(dir + "/so_residency.bin", residency);
    }
    {
      // first-order AddNoise (ParticleSystemFirstOrder.cpp:698-708): sqrt(2 D_phi) N(0,1) into omega only
      const int n = 300, s = 4;
      Thread thread(argc, argv, n, s);
      PeriodicBoundaryConditions pbc(&thread, n, s, 1.0, 1.0);
      ParticleSystemFirstOrder system(&thread, 0.3, 0.1, 1.0, 0.1, 0.2, 0.25, pbc, n, s);
      std::vector<Real> x((size_t) n * s, 0.5), derivative((size_t) n * s, 7.0), z((size_t) n);
      system.AddNoise(x, derivative, 0.0);
      unsigned long long step = 0;
      spss::check(spss_get_step_counter(system.context(), &step), "spss_get_step_counter");
      spss::check(spss_noise(system.context(), SPSS_STEPPER_STOCHASTIC_EULER, step, z.data(), (long) z.size()),
                  "spss_noise");
      system.AddNoise(x, derivative, 0.0);
      write_all(dir + "/fo_addnoise.bin", derivative);
      write_all(dir + "/fo_addnoise_z.bin", z);
    }
  } catch (const std::exception &e)
  {
    std::fprintf(stderr, "dropin_example: %s\n", e.what());
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
