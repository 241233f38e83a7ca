/*
 * A C driver of the SunlightLB API, written the way drivers of the reference
 * library are: struct fields set directly, the reference's own calls only
 * (no appended function), files written through the reference's file API.
 * It computes the drag on one sphere in a periodic box under a body force
 * (the flow through a dilute cubic array of spheres) and prints the numbers
 * with full precision, so that one source compiled against two libraries
 * (the GPU library and the CPU oracle) can be compared byte for byte.
 *
 *   sphere_drag <output directory> [steps]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sunlightlb.h"

static char *path(const char *dir, const char *name) {
  static char buf[4][1024];
  static int slot = 0;
  char *p = buf[slot++ & 3];
  snprintf(p, 1024, "%s/%s", dir, name);
  return p;
}

int main(int argc, char **argv) {
  const char *dir = argc > 1 ? argv[1] : ".";
  int steps = argc > 2 ? atoi(argv[2]) : 300, s;
  LBSys lb;
  LBObj ball;

  lb = newlb(14, 15, 16, "null");
  lb->stokes_flow = 1;
  lb->objects_moving = 0;
  lb->skip_solid = 1;
  lb->tau = 0.8;

  ball = insertsph(lb, 3.7, 6.5, 6.3, 7.2);  /* off the node lattice's symmetry centre */
  if (ball == NULL) { printf("no sphere\n"); return 1; }
  addbf(lb, 0.01, 0.0, 0.0);
  lbsavemap(lb, path(dir, "drag.map"), "list");

  for (s = 0; s < steps; s++) lbstep(lb);
  measure(lb);

  printf("step %d status %d fluid %d\n", lb->step, lb->status, countfluid(lb));
  printf("vmean %.17g %.17g %.17g\n", lb->vmeanx, lb->vmeany, lb->vmeanz);
  printf("force %.17g %.17g %.17g\n", ball->frcx, ball->frcy, ball->frcz);
  printf("torque %.17g %.17g %.17g\n", ball->trqx, ball->trqy, ball->trqz);
  printf("discrf %.17g\n", discrf(lb));

  lbsavefrc(lb, path(dir, "drag.frc"), "list");
  lbsavevel(lb, path(dir, "drag.vel"), "binary");
  lbsaveobj(lb, path(dir, "drag.obj"));
  return 0;
}
