/* gicgpu.h -- C ABI of the GB300 field-realisation library (libgicgpu.so).
 *
 * The library replaces genetIC's field-realisation hot path: white-noise drawing,
 * multiplication by sqrt(P(k)), inter-level filtering and zoom combination, the
 * modification (constraint) projections and Zel'dovich displacements/velocities.
 * genetIC's host (paramfile parser, grid geometry, particle mappers, file
 * headers and the grafIC writer) stays as it is and calls these entry points;
 * the tipsy and gadget writers' particle loops can use gic_tipsy_pack* and
 * gic_gadget_pack_host.
 *
 * Conventions (same as genetIC):
 *   - real-space index (x*N + y)*N + z, z fastest (genetIC/src/simulation/grid/grid.hpp:610-626);
 *   - Fourier fields are half spectra of N*N*(N/2+1) complex values, kz fastest,
 *     kx, ky wrapped to [0,N) (genetIC/src/tools/numerics/fourier.hpp:300-319);
 *   - both FFT directions are normalised by N^-1.5 (fourier.hpp:479-518).
 * Every call returns GIC_OK (0) or a negative status; gic_last_error() gives the
 * message.  Nothing aborts the process and no C++ exception crosses the ABI.
 * Host buffers are borrowed for the duration of a call; the context owns all
 * device memory.  Calls on one context are serialised on the context's stream
 * and have completed when they return.
 */
#ifndef GICGPU_H
#define GICGPU_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define GIC_OK 0
#define GIC_ERR_INVALID_ARG (-1)
#define GIC_ERR_OOM (-2)
#define GIC_ERR_CUDA (-3)
#define GIC_ERR_TIMEOUT (-4)
#define GIC_ERR_NOT_READY (-5)
#define GIC_ERR_INTERNAL (-6)

/* precision forms */
#define GIC_FP64 0   /* every field operation in double */
#define GIC_MIXED 1  /* FFTs and spectral multiplies in float; normalisation integral,
                        modification algebra and particle positions in double */

/* white-noise drawing modes (genetIC/src/main.cpp:44-52, ic.hpp:620-666) */
#define GIC_SEED_REAL_SPACE 0      /* random_seed_real_space / seed */
#define GIC_SEED_FOURIER_SERIAL 1  /* random_seed_serial / seedfourier */
#define GIC_SEED_FOURIER_PARALLEL 2/* random_seed / seedfourier_parallel */
#define GIC_SEED_FOURIER_REVERSE 3 /* seedfourier_reverse */

/* field selectors for gic_fetch_level / gic_fft */
#define GIC_FIELD_NOISE 0
#define GIC_FIELD_DELTA 1
#define GIC_FIELD_PSI_X 2
#define GIC_FIELD_PSI_Y 3
#define GIC_FIELD_PSI_Z 4
/* second-order (2LPT) displacements, after gic_zeldovich(ctx, 2); no genetIC counterpart */
#define GIC_FIELD_PSI2_X 5
#define GIC_FIELD_PSI2_Y 6
#define GIC_FIELD_PSI2_Z 7

#if defined(__GNUC__)
#define GIC_API __attribute__((visibility("default")))
#else
#define GIC_API
#endif

typedef struct gic_ctx gic_ctx;

typedef struct {
  int precision;     /* GIC_FP64 or GIC_MIXED */
  int device;        /* CUDA device ordinal */
  size_t mem_limit;  /* bytes of device memory the context may hold; 0 = no limit */
} gic_device_opts;

/* Cosmological parameters, as set by the paramfile commands Om, Ol, Ob, hubble,
 * s8, ns, zin (genetIC/src/main.cpp:31-37; genetIC/src/cosmology/parameters.hpp:19-32). */
typedef struct {
  double omega_m, omega_lambda, omega_b, hubble, sigma8, ns, redshift;
} gic_cosmo;

/* Context lifetime.  Replaces the state genetIC keeps in ICGenerator
 * (genetIC/src/ic.hpp:50-200). */
GIC_API int gic_create(gic_ctx **ctx, const gic_device_opts *opts);
GIC_API int gic_destroy(gic_ctx *ctx);
GIC_API const char *gic_last_error(const gic_ctx *ctx);

/* Add a grid level of n^3 cells and side `box`, lower corner (x0,y0,z0).
 * Level 0 is the periodic base grid.  Replaces MultiLevelGrid::addLevel
 * (genetIC/src/simulation/multilevelgrid/multilevelgrid.hpp:97-140) as called by
 * ICGenerator::initBaseGrid / initZoomGridWithLowLeftCornerAt (ic.hpp:502-598). */
GIC_API int gic_level_add(gic_ctx *ctx, double box, int n, double x0, double y0, double z0, int *level_id);

/* Cosmology and transfer table.  `table` is the CAMB transfer file as genetIC
 * reads it (nrows x ncols doubles, ncols 7 or 13; genetIC/src/cosmology/camb.hpp:224-268).
 * Computes the sigma8 normalisation on the device (camb.hpp:289-328).
 * Replaces CAMB<T>::CAMB (camb.hpp:195-202). */
GIC_API int gic_set_cosmology(gic_ctx *ctx, const gic_cosmo *cosmo);
GIC_API int gic_set_transfer(gic_ctx *ctx, const double *table, int nrows, int ncols);
GIC_API int gic_get_normalisation(gic_ctx *ctx, double *amplitude, double *sigma8_unnormalised);

/* Draw white noise on every level.  Reproduces RandomFieldGenerator::draw
 * (genetIC/src/simulation/field/randomfieldgenerator.hpp:122-260): GSL ranlxs2 +
 * gsl_ran_gaussian_ziggurat streams, k-shell draw order, last-write-wins folding. */
GIC_API int gic_draw_noise(gic_ctx *ctx, unsigned long seed, int mode);

/* The first n unit gaussians of the stream genetIC draws for `seed`
 * (gsl_ran_gaussian_ziggurat on a gsl_rng_ranlxs2 seeded with `seed`,
 * randomfieldgenerator.hpp:191), written to host memory.  Testing and
 * diagnostics. */
GIC_API int gic_gaussian_stream(gic_ctx *ctx, unsigned long seed, size_t n, double *host_dst);

/* Operations on the drawn white noise of every level:
 *   GIC_NOISE_REVERSE           w -> -w; ICGenerator::reverse (ic.hpp:1652-1655, multilevelfield.hpp:182-191)
 *   GIC_NOISE_REVERSE_SMALL_K   w -> -w where 0 < k^2 < param^2 (k in h/Mpc on each level's grid);
 *                               ICGenerator::reverseSmallK (ic.hpp:1690-1705)
 *   GIC_NOISE_UNIT_MODULUS      w -> w / |w|, the exact power spectrum of `fix_power`, applied by
 *                               genetIC right after drawing (ic.hpp:1342-1344, multilevelfield.hpp:395-407, 498-510) */
#define GIC_NOISE_REVERSE 0
#define GIC_NOISE_REVERSE_SMALL_K 1
#define GIC_NOISE_UNIT_MODULUS 2
GIC_API int gic_noise_op(gic_ctx *ctx, int op, double param);

/* Upload / download a level's white noise as a half spectrum of interleaved
 * (re,im) doubles.  Replaces Field data access for import_level / dump_grid_fourier. */
GIC_API int gic_set_noise(gic_ctx *ctx, int level, const double *host_src);

/* delta_k = w_k sqrt(P_grid(k)) and the Zel'dovich displacement spectra
 * psi_k = i k delta_k / k^2 on every level, then zoom combination (high-pass on
 * level l, low-passed level l-1 interpolated in) and inverse FFTs to real space.
 * Replaces ICGenerator::applyPowerSpec (ic.hpp:825-843) + OutputField::applyPowerSpectrumFor
 * (genetIC/src/simulation/field/multilevelfield.hpp:410-454) +
 * ZeldovichParticleGenerator::calculateOffsetFields (genetIC/src/simulation/particles/zeldovich.hpp:152-253)
 * + initialiseParticleGeneratorBasedOnTemplate (multilevelgenerator.hpp:78-128).
 * order: 1 = Zel'dovich (the reference's only option); 2 = second-order LPT, an
 * extension without a genetIC counterpart: psi2 = (3/7) i k S_k / k^2 with
 * S = sum_{a<b} (phi_aa phi_bb - phi_ab^2), nabla^2 phi = delta, combined across
 * levels like psi; positions q + psi + psi2, velocities ratio (psi + 2 psi2). */
GIC_API int gic_zeldovich(gic_ctx *ctx, int order);

/* Copy a level's field to the host.  Real-space fields (after gic_zeldovich)
 * are written as n^3 doubles in genetIC's (x*N+y)*N+z order; Fourier fields
 * (GIC_FIELD_NOISE) as n*n*(n/2+1) interleaved complex doubles. */
GIC_API int gic_fetch_level(gic_ctx *ctx, int level, int what, double *host_dst);

/* Particles of a level (every cell, before mapper selection): positions
 * (x,y,z interleaved, Mpc/h, wrapped into the periodic box) and velocities
 * (km/s a^1/2), as ZeldovichParticleEvaluator::getParticle evaluates them
 * (zeldovich.hpp:87-124, genetIC/src/simulation/particles/generator.hpp:49-53). */
GIC_API int gic_fetch_particles(gic_ctx *ctx, int level, double *pos, double *vel);
/* The same particles with the velocities in the precision the context computes them:
 * n^3 x 3 floats in GIC_MIXED, doubles in GIC_FP64 (positions are always doubles).
 * For callers that keep float particle arrays (genetIC's single-precision build, whose
 * ParticleEvaluator yields Particle<float>): the velocities cross the host link in half
 * the bytes, with no rounding beyond the device's own. */
GIC_API int gic_fetch_particles_native(gic_ctx *ctx, int level, double *pos, void *vel);

/* gic_fetch_particles_native without waiting: the copies are queued on the context's copy
 * stream after the work queued so far and the call returns.  pos, vel must be pinned host
 * memory and stay valid until gic_fetch_wait returns.  The next realisation of the level
 * writes its particles to a second device buffer pair while a fetch of the first may still
 * be running (a third realisation waits, on the device, for the fetch of the pair it
 * reuses), so a caller can overlap the copies of one realisation with the next one's
 * computation.  No genetIC counterpart (genetIC's evaluators return particles on demand). */
GIC_API int gic_fetch_particles_async(gic_ctx *ctx, int level, double *pos, void *vel);
/* Waits for every asynchronous fetch of the context and reports their errors. */
GIC_API int gic_fetch_wait(gic_ctx *ctx);
/* Particles of a level evaluated on a virtual grid over its region, as genetIC's
 * supersample / subsample commands produce them (SuperSampleEvaluator and
 * SubSampleEvaluator, genetIC/src/simulation/field/evaluator.hpp:96-207, over the
 * virtual grids of simulation/grid/virtualgrid.hpp:126-160, 528-605).  factor >= 2:
 * (n factor)^3 particles whose displacements are the level's, tricubic-interpolated at
 * the virtual cells' centroids (wrapped on the periodic base level, clamped on a zoom
 * level); factor <= -2: (n / |factor|)^3 particles whose displacements average each
 * block of |factor|^3 cells (|factor| must divide n).  pos, vel: (cells x 3) doubles in
 * the virtual grid's cell order, positions = centroid + displacement wrapped into the
 * box, velocities as gic_fetch_particles.  First-order (Zel'dovich) displacements. */
GIC_API int gic_fetch_particles_resampled(gic_ctx *ctx, int level, int factor, double *pos, double *vel);
/* Particles of listed cells of a zoom level's resolution-matching grid: the output grid
 * genetIC gives a zoom level when stray particles are on (strays_on; MultiLevelGrid::addLevel,
 * genetIC/src/simulation/multilevelgrid/multilevelgrid.hpp:130-137; ResolutionMatchingGrid
 * and ResolutionMatchingEvaluator, simulation/grid/virtualgrid.hpp:217-300 and
 * simulation/field/evaluator.hpp:208-256).  That grid has the level's resolution over the
 * whole region of the level above: (n_{l-1} r)^3 cells, r the cell-size ratio, cell index
 * (x m + y) m + z with m = n_{l-1} r.  Inside the zoom window a cell's particle is the
 * level's own; outside it (a stray particle) its displacement is the level above's,
 * tricubic-interpolated at the cell's centroid.  cells: n indices; pos, vel: n x 3 doubles
 * (positions wrapped into the box).  level >= 1. */
GIC_API int gic_fetch_particles_matched(gic_ctx *ctx, int level, const unsigned long long *cells, size_t n,
                                        double *pos, double *vel);

/* ---- Tipsy particle records (io::tipsy::TipsyOutput, genetIC/src/io/tipsy.hpp) ----
 * One dark-matter record, TipsyParticle::dark (tipsy.hpp:61-63). */
typedef struct {
  float mass, x, y, z, vx, vy, vz, eps, phi;
} gic_tipsy_dark;

/* The particles of a multi-level context in genetIC's mapper order
 * (OneLevelParticleMapper; TwoLevelParticleMapper nested once per zoom level, ic.hpp:1150-1185,
 * particles/mapper/twolevelmapper.hpp:262-320, 869-893): level 0's cells in cell order;
 * then for each level l >= 1, the order so far less the level-(l-1) cells in
 * replaced[l-1], followed by, for every cell of replaced[l-1] in ascending id, the
 * ratio[l]^3 level-l cells it covers, x, y, z ascending (grid.hpp:704-729).
 * replaced[l] are ascending level-l cell ids (ICGenerator's zoom masks, ic.hpp:480-569),
 * each under a replaced level-(l-1) cell; the finest level replaces none.
 * origin[l]: level l's lower corner in level-(l-1) cells.  mass and eps are each
 * level's particle mass and softening (ZeldovichParticleEvaluator::getMass/getEps),
 * and the factors TipsyOutput's (tipsy.hpp:217-239): a tipsy record holds
 * mass*mass_factor, pos*pos_factor - 0.5, vel*vel_factor, eps*pos_factor, phi = 0,
 * each product and difference rounded in double, then to float. */
#define GIC_MAP_MAX_LEVELS 8
typedef struct {
  int nlevels;                        /* 1 to GIC_MAP_MAX_LEVELS */
  int n[GIC_MAP_MAX_LEVELS];          /* cells per side (level 0 at most 1024) */
  int ratio[GIC_MAP_MAX_LEVELS];      /* ratio[l]: level-(l-1) cell size / level-l cell size */
  int origin[GIC_MAP_MAX_LEVELS][3];
  const unsigned long long *replaced[GIC_MAP_MAX_LEVELS];
  unsigned long long n_replaced[GIC_MAP_MAX_LEVELS];
  double mass[GIC_MAP_MAX_LEVELS], eps[GIC_MAP_MAX_LEVELS];
  double pos_factor, vel_factor, mass_factor;
} gic_particle_map;

/* Number of particles of the map (TwoLevelParticleMapper::size).  Without a
 * context: a failure's message is gic_last_error(NULL). */
GIC_API int gic_tipsy_count(const gic_particle_map *map, unsigned long long *count);

/* TipsyOutput's factors for the map (tipsy.hpp:200-239), ignoring the map's own factor
 * fields: the levels' masses summed one by one in mapper order, mass_factor = omega_m /
 * sum, pos_factor = 1 / box (level 0's side), vel_factor = scalefactor^-1/2 / dKmsUnit
 * with dKmsUnit = sqrt(4.3022682e-6 dMsolUnit / dKpcUnit), dKpcUnit = box 1000 / hubble,
 * dMsolUnit = 1e10 / hubble / mass_factor.  Failures: gic_last_error(NULL). */
GIC_API int gic_tipsy_factors(const gic_particle_map *map, double omega_m, double hubble, double scalefactor,
                              double box, double *pos_factor, double *vel_factor, double *mass_factor);

/* Records [first, first + count) of the map from host particles (pos[l], vel[l] for
 * every level: 3 doubles per cell in cell order, as gic_fetch_particles writes them),
 * packed by `threads` host threads (0: all cores).  Replaces the packing loop of
 * TipsyOutput::saveNextBlockOfTipsyParticles (tipsy.hpp:109-145). */
GIC_API int gic_tipsy_pack_host(const gic_particle_map *map, const double *const *pos, const double *const *vel,
                                unsigned long long first, unsigned long long count, gic_tipsy_dark *out, int threads);

/* The same records packed on the device from the context's particles (after
 * gic_zeldovich) and copied to host_out, for maps of one or two levels: 36 bytes
 * per particle cross to the host instead of the 48 of gic_fetch_particles. */
GIC_API int gic_tipsy_pack(gic_ctx *ctx, const gic_particle_map *map, unsigned long long first, unsigned long long count,
                           gic_tipsy_dark *host_out);
/* gic_tipsy_pack without waiting for the copy: the records are packed on the device and
 * their copy to host_out (pinned, valid until gic_fetch_wait returns) is queued on the
 * context's copy stream, as gic_fetch_particles_async's are; consecutive packs alternate
 * two device record buffers. */
GIC_API int gic_tipsy_pack_async(gic_ctx *ctx, const gic_particle_map *map, unsigned long long first,
                                 unsigned long long count, gic_tipsy_dark *host_out);

/* Gadget blocks (io::gadget::GadgetOutput, genetIC/src/io/gadget.hpp:481-520) of the map's
 * particles from host particles, by `threads` host threads.  level_types[l] is level l's
 * gadget particle type (0-5; gadget_particle_type, ic.hpp:606-614, 691-700); NULL means
 * type 1 for every level, genetIC's default.  The file holds the types in order, each
 * type's particles in mapper order (genericSaveBlock, gadget.hpp:285-312); [first,
 * first + count) indexes that file order.  Positions and velocities as float triples
 * (Coordinate<float> of pos and vel), ids = the particle's index in the map (the mapper
 * iterator's getIndex), masses as floats (the variable-mass block; map->mass per level).
 * NULL outputs are skipped; the map's eps and factors are not used.  Failures:
 * gic_last_error(NULL). */
GIC_API int gic_gadget_pack_host(const gic_particle_map *map, const double *const *pos, const double *const *vel,
                                 const int *level_types, unsigned long long first, unsigned long long count,
                                 float *pos_out, float *vel_out, unsigned long long *ids, float *mass_out, int threads);

/* The same gadget blocks packed on the device from the context's particles (after
 * gic_zeldovich) and copied to the host outputs, for maps of one or two levels: 40 bytes
 * per particle (all four blocks) cross to the host instead of the 48 of
 * gic_fetch_particles, and no host thread walks the mapper order.  Bit for bit the blocks
 * of gic_gadget_pack_host given the fetched particles. */
GIC_API int gic_gadget_pack(gic_ctx *ctx, const gic_particle_map *map, const int *level_types, unsigned long long first,
                            unsigned long long count, float *pos_out, float *vel_out, unsigned long long *ids,
                            float *mass_out);

/* ---- Grafic output (io::grafic::GraficOutput, genetIC/src/io/grafic.hpp:109-200) ----
 * One grid of the grafic writer's stack (copyContextWithCenteredIntermediate): a level of
 * the context (factor 1), its supersampled (factor >= 2) or subsampled (factor <= -2)
 * virtual grid, seen through a CenteredGrid when roll is non-zero: output cell (x, y, z)
 * is the grid's cell (x, y, z) - roll, periodically (roll = the CenteredGrid's integer
 * offset; 0 for the OffsetGrid-wrapped finer levels, whose cells are not moved). */
typedef struct gic_grafic_grid {
  int level;
  int factor;
  int roll[3];
  double vel_factor;            /* GraficOutput::velFactor, sqrt(a) */
  double pos_factor;            /* GraficOutput::lengthFactorDisplacements, 1 */
  unsigned long long id_offset; /* GraficOutput::iordOffset: cells of the grids written before */
} gic_grafic_grid;
/* writeGrid's per-cell values for the z-slabs [z0, z0 + nz) of that grid, as the file's
 * records hold them (each slab [y][x], x fastest): vel = 3 arrays of nz n^2 floats
 * (ic_velcx/y/z: velocity * vel_factor), pos = 3 such arrays (ic_poscx/y/z: displacement *
 * pos_factor), delta (ic_deltab: the overdensity), ids (ic_particle_ids: cell id +
 * id_offset).  NULL outputs are skipped.  The refinement mask and passive variable
 * (ic_refmap, ic_pvar_*) stay genetIC's (GraficMask).  Fields must have been computed
 * (gic_zeldovich); a virtual grid is evaluated per call, so pass all slabs at once. */
GIC_API int gic_grafic_pack(gic_ctx *ctx, const gic_grafic_grid *grid, int z0, int nz, float *vel, float *pos,
                            float *delta, unsigned long long *ids);

/* Forward (dir=-1) or inverse (dir=+1) normalised 3-D real FFT of a level field
 * in place on the device (testing).  Replaces FieldFourierManager<T,T>::performTransform
 * (fourier.hpp:479-518). */
GIC_API int gic_fft(gic_ctx *ctx, int level, int what, int dir);

/* gic_fft restricted to a box of the level's cells: per axis a the cyclic range
 * start[a] .. start[a] + len[a] - 1 (mod n).  dir = -1: the real field must be zero
 * outside the box (the padding words of the rows need not be); dir = +1: only the
 * real values inside the box are defined afterwards.  Inside the box the values are
 * the bits gic_fft gives; the transforms skip the x planes and y rows outside it.
 * No genetIC counterpart: FFTW plans always transform the whole grid. */
GIC_API int gic_fft_box(gic_ctx *ctx, int level, int what, int dir, const int *start, const int *len);

/* chi^2 of the white noise <C^-1 w | w>: Hermitian-weighted sum of |w_k|^2 on
 * one level; with zoom levels the covariance metric with windowed filters
 * (MultiLevelField::getChi2, multilevelfield.hpp:461-487, 344-384). */
GIC_API int gic_chi2(gic_ctx *ctx, double *chi2);

/* modification kinds (genetIC/src/simulation/modifications/modificationmanager.hpp:160-192) */
#define GIC_MOD_OVERDENSITY 0
#define GIC_MOD_VX 1
#define GIC_MOD_VY 2
#define GIC_MOD_VZ 3
#define GIC_MOD_POTENTIAL 4 /* PotentialModification (linearmodification.hpp:146-169) */
#define GIC_MOD_LX 5        /* AngMomentumModification (linearmodification.hpp:300-412), x, y, z */
#define GIC_MOD_LY 6
#define GIC_MOD_LZ 7

/* Current value <a|w> of a modification's quantity (mean overdensity, or mean
 * velocity component, over `cells`, the flagged cells of the finest level as
 * linear indices) on the white noise.  Replaces
 * ModificationManager::calculateCurrentValueByName (modificationmanager.hpp:37-45). */
GIC_API int gic_calculate(gic_ctx *ctx, int kind, const unsigned long long *cells, size_t n, double *value);

/* Queue a linear modification: absolute target, or relative (target times the
 * current value).  Replaces ModificationManager::addModificationToList
 * (modificationmanager.hpp:59-82). */
GIC_API int gic_add_modification(gic_ctx *ctx, int kind, const unsigned long long *cells, size_t n, double target,
                                 int relative);
GIC_API int gic_clear_modifications(gic_ctx *ctx);

/* Splicing: replace the white noise on each level's flagged cells (cells[l], as
 * for the variance) by a new real-space draw of `new_seed`, keeping the rest as
 * close to the original as the covariance allows: spliceOneLevel's preconditioned
 * conjugate-gradient solve per level (modifications/splice.hpp:37-118,
 * tools/numerics/cg.hpp:13-59, ICGenerator::splice ic.hpp:1658-1688), including the
 * reference's inner products over its whole transform buffers.  iterations[l]
 * (optional) receives each level's CG iterations. */
GIC_API int gic_splice(gic_ctx *ctx, unsigned long new_seed, const unsigned long long *const *cells,
                       const size_t *counts, int *iterations);

/* Quadratic modification: the variance, over the flagged cells of each level, of
 * the dark-matter overdensity high-passed at `filterscale` (Mpc/h; the filter is
 * 1 - a Fermi low-pass at k = 2 pi / filterscale).  `cells[l]` / `counts[l]` hold
 * the flagged cells of level l as sorted linear indices, one array per level.
 * Replaces FilteredVarianceModification::calculateCurrentValue
 * (quadraticmodification.hpp:51-57, 118-221) reached through
 * ModificationManager::calculateCurrentValueByName (modificationmanager.hpp:37-45).
 * Fails with GIC_ERR_INVALID_ARG when filterscale is negative (never set) or
 * below the finest cell size, as checkFilterScale (quadraticmodification.hpp:131-153). */
GIC_API int gic_calculate_variance(gic_ctx *ctx, const unsigned long long *const *cells, const size_t *counts,
                                   double filterscale, double *value);

/* Queue a variance modification (absolute, or relative to its current value).
 * gic_apply_modifications applies it after the linear ones by the reference's
 * iterative scheme: a trial of `init_steps` steps on a copy fixes the number of
 * steps from `precision` (modificationmanager.hpp:221-285; genetIC uses 10 and
 * 0.001, ic.hpp:160-161).  Replaces ModificationManager::addModificationToList for
 * "variance" (modificationmanager.hpp:59-82, 188-196). */
GIC_API int gic_add_variance_modification(gic_ctx *ctx, const unsigned long long *const *cells, const size_t *counts,
                                          double filterscale, double target, int relative, int init_steps,
                                          double precision);

/* ---- Gradients through the realisation (no genetIC counterpart) -------------
 * For the Python autograd binding.  Arrays are DEVICE pointers in the context's
 * precision (float for GIC_MIXED, double for GIC_FP64), compact n^3 per level in
 * genetIC's (x n + y) n + z order.  A level's white noise is taken as its real
 * field w (unit gaussians), the inverse unitary transform of the half spectrum
 * the reference draws.  Calls run on the context's stream and return when done.
 * Gradients through the zoom combination are available for levels 0 and 1. */

/* The drawn white noise of a level as a real field. */
GIC_API int gic_noise_real(gic_ctx *ctx, int level, void *dev_out);

/* `what` (GIC_FIELD_DELTA or GIC_FIELD_PSI_X..Z) of `level` from the real white
 * noise of every level (dev_noise[l]), as gic_zeldovich forms it (own level times
 * sqrt(P) and its high-pass; on level 1 plus the base level's low-passed field
 * interpolated in), and its adjoint: dev_grad_noise[l] = (d field / d w_l)^T g. */
GIC_API int gic_field_from_noise(gic_ctx *ctx, int level, int what, const void *const *dev_noise, void *dev_out);
GIC_API int gic_field_from_noise_adjoint(gic_ctx *ctx, int level, int what, const void *dev_grad_out,
                                         void *const *dev_grad_noise);

/* The variance functional <A w|w> of gic_calculate_variance at the real white
 * noise dev_noise[l] (A w = the pushed covector, quadraticmodification.hpp:59-92),
 * and its gradient in dev_grad[l]: with `exact`, (A + A^T) w through the
 * transposed kernels; otherwise 2 A w, the direction of the reference's quadratic
 * solver (modificationmanager.hpp:249-275).  The two agree on one level; across
 * levels the covector metric's cross terms make A unsymmetric. */
GIC_API int gic_variance_gradient(gic_ctx *ctx, const unsigned long long *const *cells, const size_t *counts,
                                  double filterscale, const void *const *dev_noise, void *const *dev_grad,
                                  int exact, double *value);

/* Apply the queued modifications to the white noise (orthonormalised, with the
 * covariance metric), returning chi^2 before and after.  Replaces
 * ModificationManager::applyModifications (modificationmanager.hpp:90-125). */
GIC_API int gic_apply_modifications(gic_ctx *ctx, double *chi2_before, double *chi2_after);

/* Allocation-free variant of gic_gaussian_stream.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc (for instance
 * code that must stay inside another runtime's device-memory pool or budget).
 * Writes the first n unit gaussians of the stream of `seed` to the caller's
 * device buffer `device_out` (n doubles) on the caller's CUDA stream `stream`
 * (a cudaStream_t, NULL = legacy default stream).  The call reads a status
 * flag back and synchronises `stream` before it returns.  It allocates
 * nothing: its scratch is one file-scope device array of 24 MiB that every
 * device loading the library holds until the process exits.  n may be at most
 * GIC_NOALLOC_MAX_GAUSSIANS; larger n returns GIC_ERR_INVALID_ARG without
 * touching the GPU.  The first call on each device (and in each new CUDA
 * context of it) looks up the array's device address, so make that call before
 * any stream capture.  All calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller.  Errors are status codes only (no
 * message). */
#define GIC_NOALLOC_MAX_GAUSSIANS (1ull << 20)
GIC_API int gic_gaussian_stream_noalloc(unsigned long seed, size_t n, double *device_out, void *stream);

/* ---- Batches of independent realisations on one GPU (no genetIC counterpart) ----
 * A batch groups contexts of one device (any sizes, levels and modifications).
 * gic_batch_realise realises every context: white noise (seeds[i], seeding mode
 * modes[i], or the parallel Fourier mode when modes is NULL), its queued
 * modifications, fields and particles (order 1 or 2), each context on its own
 * stream.  Contexts whose modifications are all linear (at most 16) are realised
 * by one CUDA graph over all of them, captured on the first call (after an eager
 * realisation) and replayed on later calls while the contexts' buffers, seeding
 * modes, order and modification targets stay the same; it is captured again when
 * any changed.  Contexts with a variance modification are realised from `threads`
 * host threads beside it.  Returns when all realisations are complete; results
 * are then read per context. */
typedef struct gic_batch gic_batch;
GIC_API int gic_batch_create(gic_batch **out, gic_ctx *const *ctxs, int n);
GIC_API int gic_batch_destroy(gic_batch *batch);
GIC_API int gic_batch_realise(gic_batch *batch, const unsigned long *seeds, const int *modes, int order, int threads);
GIC_API const char *gic_batch_last_error(const gic_batch *batch);
/* The stream a batch's graph runs on; every realisation of gic_batch_realise is
 * ordered between work queued on it before the call and work queued after. */
GIC_API int gic_batch_get_stream(gic_batch *batch, void **stream);
/* The batch's graph: the contexts it realises, the kernels of one replay, the
 * replays since it was captured, and (empty unless) why the batch stopped
 * capturing.  Any pointer may be NULL. */
GIC_API int gic_batch_graph_info(const gic_batch *batch, int *contexts, unsigned long long *kernels, int *replays,
                                 const char **off_reason);

/* Number of kernels this library has launched in the process so far. */
GIC_API int gic_launch_count(unsigned long long *count);

/* The bounded waits of the FFT plane pass (a persistent kernel whose CTAs wait, one
 * thread each, for tiles other CTAs of the launch write: the L2-resident fusion of a
 * transform's y and z passes).  Each wait polls at most spin_limit times, 100 ns apart
 * (0 = the default, 2^22: about 0.4 s), then gives up, flags it and carries on, so the
 * kernel always ends; the call then returns GIC_ERR_TIMEOUT and the transform's
 * results are invalid.  unreachable != 0 (tests only) sets every wait a target no
 * task can reach, so each one gives up after spin_limit polls.  No counterpart in
 * genetIC (its FFTW transforms have no waits). */
GIC_API int gic_set_fft_wait(gic_ctx *ctx, unsigned spin_limit, int unreachable);

/* The FFT passes the context uses for n^3 transforms in its precision (chosen by timing
 * the candidates on first use, or pinned by GIC_FFT_TILE=<cols>,<rows>[,<plane variant>]):
 * strided-pass candidate (6: TMA-staged), row-pass candidate and plane-pass variant (-1:
 * separate y and z passes).  GIC_ERR_NOT_READY before the first n^3 transform, or when
 * n^3 uses the runtime-length passes.  The choice never changes a result. */
GIC_API int gic_fft_choice(gic_ctx *ctx, int n, int *cols, int *rows, int *planes);

/* Device memory the context holds now, in bytes, and its mem_limit (0 = none).
 * Every device allocation a call makes for the context is checked against the limit
 * first: one that would pass it fails the call with GIC_ERR_OOM (the message names
 * the sizes) and allocates nothing; the context stays usable, and later calls that
 * fit run normally.  genetIC has no counterpart: its fields live in host memory. */
GIC_API int gic_memory_use(gic_ctx *ctx, size_t *in_use, size_t *limit);

/* The context's CUDA stream (a cudaStream_t), for callers that order their own
 * work or timing events after the library's. */
GIC_API int gic_get_stream(gic_ctx *ctx, void **stream);

#ifdef __cplusplus
}
#endif
#endif
