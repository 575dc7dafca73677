// Compile check of the genetIC-side hook (include/gicgpu_genetic.hpp) against genetIC's
// own headers: instantiates the device-backed evaluator and the realisation context for
// genetIC's double (FP64) and float (-f, mixed precision) builds.  Built by oracle/Makefile's
// `hook` target where genetIC's sources are; nothing here runs.
// genetIC's main.cpp includes, in its order, then the hook
#include <stdlib.h>
#include <sstream>
#include <ctime>
#include <iostream>
#include <iomanip>
#include "src/tools/parser.hpp"
#include "src/tools/logging.hpp"
#include "src/ic.hpp"
#include "gicgpu_genetic.hpp"

template class gicgpu::DeviceRealisation<double>;
template class gicgpu::DeviceRealisation<float>;
template class gicgpu::DeviceBackedParticleEvaluator<double>;
template class gicgpu::DeviceBackedParticleEvaluator<float>;

// the writer's view: a ParticleEvaluator, as io/tipsy.hpp and io/gadget.hpp take it
std::shared_ptr<particle::ParticleEvaluator<double>> device_evaluator(const grids::Grid<double> &g,
                                                                    const cosmology::CosmologicalParameters<double> &c,
                                                                    gicgpu::DeviceRealisation<double> &gpu, int level) {
  std::vector<double> pos, vel;
  gpu.fetchParticles(level, g.size3, pos, vel);
  return std::make_shared<gicgpu::DeviceBackedParticleEvaluator<double>>(g, c, std::move(pos), std::move(vel));
}
