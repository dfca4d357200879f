/*
 * Test driver for the C adapter of INTEGRATION.md (tests/test_integration_adapter.py).
 *
 * Compiled together with the adapter against the reference's own headers
 * (src/meraxes.h: run_globals_t, reion_grids_t, ABORT) and linked with
 * libmxreion.so.  It fills run_globals for a small box the way
 * init_meraxes() does for the fields the adapter reads, allocates the grids
 * in the reference layouts, and calls the three entry points the adapter
 * exports: ComputeTs(), find_HII_bubbles(), ComputeBrightnessTemperatureBox().
 *
 * Exit status: 0 when the three calls return; ABORT (an adapter error, e.g.
 * no CUDA device) goes through myexit(), which exits with 3.
 */
#define _MAIN
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "meraxes.h"

#include "BrightnessTemperature.h"
#include "ComputeTs.h"
#include "find_HII_bubbles.h"

void myexit(int signum)
{
  fprintf(stderr, "adapter_drive: ABORT(%d)\n", signum);
  exit(3);
}

static float* grid(size_t n, float v)
{
  float* g = (float*)malloc(sizeof(float) * n);
  for (size_t i = 0; i < n; i++)
    g[i] = v;
  return g;
}

int main(int argc, char** argv)
{
  const int D = 16;
  const size_t real = (size_t)D * D * D, padded = (size_t)D * D * 2 * (D / 2 + 1);
  memset(&run_globals, 0, sizeof(run_globals));
  run_params_t* rp = &run_globals.params;
  physics_params_t* ph = &rp->physics;
  rp->BoxSize = 25.0;
  rp->Hubble_h = 0.678;
  rp->OmegaM = 0.308;
  rp->OmegaLambda = 0.692;
  rp->BaryonFrac = 0.157;
  rp->wLambda = -1.0;
  rp->ReionGridDim = D;
  rp->ReionDeltaRFactor = 1.1;
  rp->TsNumFilterSteps = 40;
  rp->ReionSfrTimescale = 0.5;
  rp->Flag_IncludeSpinTemp = 1;
  rp->Flag_IncludeRecombinations = 1;
  rp->Flag_Compute21cmBrightTemp = 1;
  rp->ReionUVBFlag = 1;
  rp->SnaplistLength = 2;
  strncpy(rp->TablesForXHeatingDir, argc > 1 ? argv[1] : ".", STRLEN - 1);
  ph->ReionEfficiency = 1.0;
  ph->ReionNionPhotPerBary = 4000.0;
  ph->ReionGammaHaloBias = 2.0;
  ph->ReionAlphaUV = 5.0;
  ph->Y_He = 0.24;
  ph->ReionRBubbleMin = 0.0;
  ph->ReionRBubbleMax = 20.0;
  ph->ReionRBubbleMaxRecomb = 20.0;
  ph->ReionMaxHeatingRedshift = 35.0;
  ph->LXrayGal = 1e40;
  ph->NuXrayGalThreshold = 500.0;
  ph->SpecIndexXrayGal = 1.0;
  ph->NuXraySoftCut = 2000.0;
  ph->NuXrayMax = 10000.0;
  run_globals.units.UnitLength_in_cm = 3.08568e24;
  run_globals.units.UnitMass_in_g = 1.989e43;
  run_globals.units.UnitVelocity_in_cm_per_s = 1e5;
  static double zz[2] = { 10.5, 10.0 };
  run_globals.ZZ = zz;

  reion_grids_t* g = &run_globals.reion_grids;
  g->deltax = grid(padded, 0.1f);
  g->stars = grid(padded, 0.0f);
  g->weighted_sfr = grid(padded, 0.0f);
  g->sfr = grid(padded, 0.0f);
  g->sfr_histories = grid(padded * 8, 0.0f);
  g->N_rec = grid(padded, 0.0f);
  g->x_e_box = grid(padded, 1e-4f);
  g->x_e_box_prev = grid(padded, 1e-4f);
  g->Tk_box = grid(real, 10.0f);
  g->TS_box = grid(real, 10.0f);
  g->xH = grid(real, 1.0f);
  g->z_at_ionization = grid(real, -1.0f);
  g->r_bubble = grid(real, 0.0f);
  g->J_21 = grid(real, 0.0f);
  g->J_21_at_ionization = grid(real, 0.0f);
  g->Gamma12 = grid(real, 0.0f);
  g->delta_T = grid(real, 0.0f);

  ComputeTs(1, NULL);
  find_HII_bubbles(1, NULL);
  ComputeBrightnessTemperatureBox(1);
  printf("adapter_drive: xH %.9g TS %.9g Tb %.9g\n", g->volume_weighted_global_xH, g->volume_ave_TS,
         g->volume_ave_Tb);
  return 0;
}
