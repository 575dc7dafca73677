/* A plain C caller of libgicgpu.so: one FP64 Zel'dovich realisation of a 32^3 grid in a
 * 50 Mpc/h box (serial Fourier seeding, the cosmology given on the command line's table),
 * written out as raw doubles: the overdensity (32^3), then positions and velocities
 * (3 x 32^3 each).  Usage: realise32 <transfer table: nrows x 7 doubles> <nrows> <out>.
 * Exits 0 on success; on a failing call prints the library's message and exits 1. */
#include <stdio.h>
#include <stdlib.h>

#include "gicgpu.h"

#define N 32

static gic_ctx *ctx;

static void check(int status, const char *what) {
  if (status != GIC_OK) {
    fprintf(stderr, "%s failed (%d): %s\n", what, status, gic_last_error(ctx));
    exit(1);
  }
}

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s table.bin nrows out.bin\n", argv[0]);
    return 2;
  }
  const int nrows = atoi(argv[2]);
  double *table = malloc(sizeof(double) * 7 * (size_t)nrows);
  FILE *f = fopen(argv[1], "rb");
  if (!f || !table || fread(table, sizeof(double), 7 * (size_t)nrows, f) != 7 * (size_t)nrows) return 2;
  fclose(f);

  gic_device_opts opts = {GIC_FP64, 0, 0};
  if (gic_create(&ctx, &opts) != GIC_OK) {
    fprintf(stderr, "gic_create: %s\n", gic_last_error(NULL));
    return 1;
  }
  gic_cosmo cosmo = {0.31, 0.69, 0.0, 0.68, 0.81, 0.965, 99.0};
  int level = -1;
  check(gic_set_cosmology(ctx, &cosmo), "gic_set_cosmology");
  check(gic_set_transfer(ctx, table, nrows, 7), "gic_set_transfer");
  check(gic_level_add(ctx, 50.0, N, 0.0, 0.0, 0.0, &level), "gic_level_add");
  check(gic_draw_noise(ctx, 8896131ul, GIC_SEED_FOURIER_SERIAL), "gic_draw_noise");
  check(gic_zeldovich(ctx, 1), "gic_zeldovich");
  const size_t m = (size_t)N * N * N;
  double *delta = malloc(sizeof(double) * m), *pos = malloc(sizeof(double) * 3 * m), *vel = malloc(sizeof(double) * 3 * m);
  if (!delta || !pos || !vel) return 1;
  check(gic_fetch_level(ctx, level, GIC_FIELD_DELTA, delta), "gic_fetch_level");
  check(gic_fetch_particles(ctx, level, pos, vel), "gic_fetch_particles");
  /* a refused call: an unknown field leaves the context as it was */
  if (gic_fetch_level(ctx, level, 999, delta) != GIC_ERR_INVALID_ARG) {
    fprintf(stderr, "an unknown field was not refused\n");
    return 1;
  }
  check(gic_destroy(ctx), "gic_destroy");
  FILE *o = fopen(argv[3], "wb");
  if (!o) return 1;
  fwrite(delta, sizeof(double), m, o);
  fwrite(pos, sizeof(double), 3 * m, o);
  fwrite(vel, sizeof(double), 3 * m, o);
  fclose(o);
  free(delta);
  free(pos);
  free(vel);
  free(table);
  return 0;
}
