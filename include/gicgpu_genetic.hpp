// The genetIC side of the drop-in: C++ over the C ABI of gicgpu.h, written against
// genetIC's own types, for a genetIC build with -DGIC_GPU.  genetIC's headers rely on
// the includes of its main.cpp, so this header is included after genetIC's ic.hpp (at
// the end of its includes, or in main.cpp after it).  It replaces the field-realisation
// path behind genetIC's unchanged parser, mappers and writers:
//
//   gicgpu::DeviceRealisation  one context: the cosmology and transfer table of
//                              ICGenerator::setCambDat (genetIC/src/ic.hpp:725-728), the levels
//                              of addLevelToContext (ic.hpp:606-614), the white noise of
//                              initialiseAllRandomComponents (ic.hpp:1334-1352) and the
//                              Zel'dovich particles that write (ic.hpp:1275-1331) evaluates
//   gicgpu::DeviceBackedParticleEvaluator
//                              a particle::ParticleEvaluator
//                              (genetIC/src/simulation/particles/generator.hpp:17-54) over the
//                              positions and velocities fetched from the device, giving the
//                              masses and softenings ZeldovichParticleEvaluator gives
//                              (genetIC/src/simulation/particles/zeldovich.hpp:53-124), so the
//                              writers and mappers read it unchanged.
//
// Every failing call throws std::runtime_error with the library's message; genetIC's
// dispatcher reports it with the paramfile line (genetIC/src/tools/parser.hpp:204-207).
#pragma once
#include <cmath>
#include <complex>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "gicgpu.h"

namespace gicgpu {

inline void check(gic_ctx *ctx, int status, const char *what) {
  if (status != GIC_OK)
    throw std::runtime_error(std::string("gicgpu: ") + what + ": " + (ctx ? gic_last_error(ctx) : "no context"));
}

// One realisation context on one GPU.  T is genetIC's coordinate type: float builds
// (genetIC -f) take the mixed-precision form, double builds the FP64 form.
template <typename T>
class DeviceRealisation {
  gic_ctx *ctx_ = nullptr;

 public:
  explicit DeviceRealisation(int device = 0, size_t mem_limit = 0) {
    gic_device_opts o{std::is_same<T, float>::value ? GIC_MIXED : GIC_FP64, device, mem_limit};
    if (gic_create(&ctx_, &o) != GIC_OK) throw std::runtime_error("gicgpu: no context: " + std::string(gic_last_error(nullptr)));
  }
  ~DeviceRealisation() { gic_destroy(ctx_); }
  DeviceRealisation(const DeviceRealisation &) = delete;
  DeviceRealisation &operator=(const DeviceRealisation &) = delete;
  gic_ctx *context() const { return ctx_; }

  // setCambDat: genetIC's cosmology, then the CAMB table it read
  // (io::getBufferIgnoringColumnHeaders: rows of 7 or 13 columns)
  void setCosmology(const cosmology::CosmologicalParameters<T> &c) {
    gic_cosmo g{(double)c.OmegaM0, (double)c.OmegaLambda0, (double)c.OmegaBaryons0, (double)c.hubble,
                (double)c.sigma8, (double)c.ns, (double)c.redshift};
    check(ctx_, gic_set_cosmology(ctx_, &g), "gic_set_cosmology");
  }
  void setTransfer(const std::vector<double> &table, int ncols) {
    check(ctx_, gic_set_transfer(ctx_, table.data(), (int)(table.size() / ncols), ncols), "gic_set_transfer");
  }

  // addLevelToContext: a grid of the multi-level context, coarsest first
  int addLevel(const grids::Grid<T> &g) {
    int id = -1;
    check(ctx_, gic_level_add(ctx_, (double)g.thisGridSize, (int)g.size, (double)g.offsetLower.x,
                              (double)g.offsetLower.y, (double)g.offsetLower.z, &id),
          "gic_level_add");
    return id;
  }

  // initialiseAllRandomComponents: the seed and the mode setSeed* chose
  void drawNoise(unsigned long seed, int mode) { check(ctx_, gic_draw_noise(ctx_, seed, mode), "gic_draw_noise"); }

  // modify / calculate on the finest level's flagged cells (getFlaggedCells)
  void addModification(int kind, const std::vector<size_t> &cells, double target, int relative) {
    std::vector<unsigned long long> c(cells.begin(), cells.end());
    check(ctx_, gic_add_modification(ctx_, kind, c.data(), c.size(), target, relative), "gic_add_modification");
  }
  double calculate(int kind, const std::vector<size_t> &cells) {
    std::vector<unsigned long long> c(cells.begin(), cells.end());
    double v = 0;
    check(ctx_, gic_calculate(ctx_, kind, c.data(), c.size(), &v), "gic_calculate");
    return v;
  }
  void applyModifications(double &chi2_before, double &chi2_after) {
    check(ctx_, gic_apply_modifications(ctx_, &chi2_before, &chi2_after), "gic_apply_modifications");
  }

  // write: the particles of every level (order 1: Zel'dovich, as genetIC; 2: 2LPT)
  void realise(int order = 1) { check(ctx_, gic_zeldovich(ctx_, order), "gic_zeldovich"); }
  void fetchParticles(int level, size_t ncells, std::vector<double> &pos, std::vector<double> &vel) {
    pos.resize(3 * ncells);
    vel.resize(3 * ncells);
    check(ctx_, gic_fetch_particles(ctx_, level, pos.data(), vel.data()), "gic_fetch_particles");
  }
  // dump_grid: the level's overdensity, n^3 doubles in genetIC's (x n + y) n + z order
  void fetchOverdensity(int level, size_t ncells, std::vector<double> &out) {
    out.resize(ncells);
    check(ctx_, gic_fetch_level(ctx_, level, GIC_FIELD_DELTA, out.data()), "gic_fetch_level");
  }
};

// The particles of one level, read from host copies of the device's positions (wrapped
// into the box) and velocities.  Masses and softenings are ZeldovichParticleEvaluator's:
// 27.744948 Omega_m L^3 times the cell's mass fraction, and cellSize * cellSofteningScale
// * epsNorm.
template <typename GridDataType, typename T = tools::datatypes::strip_complex<GridDataType>>
class DeviceBackedParticleEvaluator : public particle::ParticleEvaluator<GridDataType> {
  std::vector<double> pos_, vel_;
  T boxMass_, epsNorm_, smoothNorm_;
  std::shared_ptr<const grids::Grid<T>> onGrid_;

 public:
  DeviceBackedParticleEvaluator(const grids::Grid<T> &grid, const cosmology::CosmologicalParameters<T> &cosmology,
                                std::vector<double> pos, std::vector<double> vel, T epsNorm = 0.01075)
      : particle::ParticleEvaluator<GridDataType>(grid), pos_(std::move(pos)), vel_(std::move(vel)),
        boxMass_(T(27.744948) * cosmology.OmegaM0 * std::pow(grid.periodicDomainSize, T(3))), epsNorm_(epsNorm),
        smoothNorm_(cosmology.smoothNorm), onGrid_(grid.shared_from_this()) {
    if (pos_.size() != 3 * grid.size3 || vel_.size() != 3 * grid.size3)
      throw std::runtime_error("gicgpu: particle arrays do not match the grid");
  }

  particle::Particle<T> getParticleNoWrap(size_t id) const override {
    particle::Particle<T> p;
    p.pos = Coordinate<T>(T(pos_[3 * id]), T(pos_[3 * id + 1]), T(pos_[3 * id + 2]));
    p.vel = Coordinate<T>(T(vel_[3 * id]), T(vel_[3 * id + 1]), T(vel_[3 * id + 2]));
    p.mass = getMass();
    p.soft = getEps();
    return p;
  }

  // the displacement: the position less the cell's centroid, taken to the nearest image
  particle::Particle<T> getParticleNoOffset(size_t id) const override {
    particle::Particle<T> p = getParticleNoWrap(id);
    const Coordinate<T> c = onGrid_->getCentroidFromIndex(id);
    const T L = onGrid_->periodicDomainSize;
    auto nearest = [L](T d) { return d - L * std::round(d / L); };
    p.pos = Coordinate<T>(nearest(p.pos.x - c.x), nearest(p.pos.y - c.y), nearest(p.pos.z - c.z));
    return p;
  }

  T getMass() const override { return boxMass_ * onGrid_->cellMassFrac; }
  T getEps() const override { return onGrid_->cellSize * onGrid_->cellSofteningScale * epsNorm_; }
  T getSmoothingScale() const override { return onGrid_->cellSize * smoothNorm_; }
};

}  // namespace gicgpu
