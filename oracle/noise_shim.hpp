/*
 * Noise-replay shim, force-included (g++ -include) when the reference's own
 * sources are compiled as the CPU oracle.  Test infrastructure only.
 *
 * The reference draws every Gaussian through
 *     std::normal_distribution<Real> norm_dist(0.0, 1.0);
 *     norm_dist(mersenne_twister_generator);
 * (Steppers/StochasticRungeKuttaStepperPtr.hpp:50,54,
 *  Steppers/StochasticEulerStepperPtr.hpp:49,56,85,92-94,
 *  DynamicalSystems/ParticleSystemSecondOrder.cpp:443,447-449).
 * After <random> is included, `normal_distribution` is redefined to a
 * distribution that ignores the generator and returns the next value of a
 * replay buffer filled by ref_driver.cpp.  The GPU writes that buffer from the
 * exact normals its Philox stream produced, so the oracle and the GPU see
 * identical noise in the reference's draw order.
 *
 * The replacement template is declared inside namespace std because the
 * reference spells the type `std::normal_distribution`.  Adding a name to
 * std is formally undefined behaviour; GCC accepts it, and this header is
 * never part of the product.
 */
#ifndef SPSS_ORACLE_NOISE_SHIM_HPP
#define SPSS_ORACLE_NOISE_SHIM_HPP

#include <random>

namespace spss_replay
{
double next();
}

namespace std
{
template<class RealType = double>
class spss_replay_normal_distribution
{
 public:
  explicit spss_replay_normal_distribution(RealType = RealType(0), RealType = RealType(1))
  {}
  template<class Generator>
  RealType operator()(Generator &)
  {
    return static_cast<RealType>(spss_replay::next());
  }
};
}

#define normal_distribution spss_replay_normal_distribution

#endif
