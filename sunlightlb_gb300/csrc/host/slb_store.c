/*
 * Checkpoint and field I/O (reference src/lbstore.c) and signal handling
 * (reference src/lbsignal.c).  File formats are byte-compatible with the
 * reference: moments and forces as LBStoreReal, velocity files as LBReal
 * (binary) or text.  Populations are read back from the GPU for saving; the
 * velocity warm start rebuilds populations on the GPU.
 */
#include <signal.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include "slb_private.h"

/* moments of one node's populations, reference src/lbstore.c:61-74 */
static void moments(const LBReal *t, LBReal m[10]) {
  LBReal p12 = t[1] + t[2], p34 = t[3] + t[4], p56 = t[5] + t[6];
  LBReal lo_sum = t[7] + t[8] + t[9] + t[10], hi_sum = t[11] + t[12] + t[13] + t[14];
  LBReal lo_x = t[7] - t[8] + t[9] - t[10], hi_x = t[11] - t[12] + t[13] - t[14];
  LBReal lo_y = t[7] + t[8] - t[9] - t[10], hi_y = t[11] + t[12] - t[13] - t[14];
  LBReal lo_xy = t[7] - t[8] - t[9] + t[10], hi_xy = t[11] - t[12] - t[13] + t[14];
  LBReal p06 = t[0] + p12 + p34 + p56, twoby3 = 2.0 / 3.0, sdiag;
  m[0] = p06 + (lo_sum + hi_sum);
  m[1] = t[1] - t[2] + lo_x + hi_x;
  m[2] = t[3] - t[4] + lo_y + hi_y;
  m[3] = t[5] - t[6] + lo_sum - hi_sum;
  sdiag = twoby3 * m[0] - p06;
  m[4] = sdiag + p12; m[5] = sdiag + p34; m[6] = sdiag + p56;
  m[7] = lo_xy + hi_xy; m[8] = lo_x - hi_x; m[9] = lo_y - hi_y;
}

/* moments as lbsave stores them: drho is rounded to LBStoreReal before the
 * stress is formed from it (reference src/lbstore.c:42, 68-74) */
static void store_moments(const LBReal *t, LBStoreReal m[10]) {
  LBReal p12 = t[1] + t[2], p34 = t[3] + t[4], p56 = t[5] + t[6];
  LBReal lo_sum = t[7] + t[8] + t[9] + t[10], hi_sum = t[11] + t[12] + t[13] + t[14];
  LBReal lo_x = t[7] - t[8] + t[9] - t[10], hi_x = t[11] - t[12] + t[13] - t[14];
  LBReal lo_y = t[7] + t[8] - t[9] - t[10], hi_y = t[11] + t[12] - t[13] - t[14];
  LBReal lo_xy = t[7] - t[8] - t[9] + t[10], hi_xy = t[11] - t[12] - t[13] + t[14];
  LBReal p06 = t[0] + p12 + p34 + p56, twoby3 = 2.0 / 3.0, sdiag;
  m[0] = p06 + (lo_sum + hi_sum);
  m[1] = t[1] - t[2] + lo_x + hi_x;
  m[2] = t[3] - t[4] + lo_y + hi_y;
  m[3] = t[5] - t[6] + lo_sum - hi_sum;
  sdiag = twoby3 * m[0] - p06;
  m[4] = sdiag + p12; m[5] = sdiag + p34; m[6] = sdiag + p56;
  m[7] = lo_xy + hi_xy; m[8] = lo_x - hi_x; m[9] = lo_y - hi_y;
}

/* populations from stored moments with the reference's mixed float/double
 * evaluation (reference src/lbstore.c:106-109, 145-203) */
static void rebuild_store(LBReal *t, LBStoreReal drho, LBStoreReal rux, LBStoreReal ruy,
                          LBStoreReal ruz, LBStoreReal sxx, LBStoreReal syy, LBStoreReal szz,
                          LBStoreReal sxy, LBStoreReal sxz, LBStoreReal syz, int average) {
  LBReal b = 72.0, dbybc2 = 1.0 / 24.0, dd2bybc4 = 1.0 / 8.0;
  LBReal fdd2bybc4 = 4.0 * dd2bybc4, edbybc2 = 8.0 * dbybc2;
  LBReal rhobyb = drho / b, erhobyb = 8.0 * rhobyb, trsby3 = (sxx + syy + szz) / 3.0, ru, st, v[15];
  int q;
  v[0] = 2.0 * erhobyb - 2.0 * fdd2bybc4 * trsby3;
  ru = edbybc2 * rux; st = fdd2bybc4 * (sxx - trsby3);
  v[1] = erhobyb + ru + st; v[2] = erhobyb - ru + st;
  ru = edbybc2 * ruy; st = fdd2bybc4 * (syy - trsby3);
  v[3] = erhobyb + ru + st; v[4] = erhobyb - ru + st;
  ru = edbybc2 * ruz; st = fdd2bybc4 * (szz - trsby3);
  v[5] = erhobyb + ru + st; v[6] = erhobyb - ru + st;
  ru = dbybc2 * (rux + ruy + ruz); st = dd2bybc4 * (trsby3 + sxy + sxz + syz);
  v[7] = rhobyb + ru + st; v[14] = rhobyb - ru + st;
  ru = dbybc2 * (rux - ruy - ruz); st = dd2bybc4 * (trsby3 - sxy - sxz + syz);
  v[8] = rhobyb - ru + st; v[13] = rhobyb + ru + st;
  ru = dbybc2 * (rux - ruy + ruz); st = dd2bybc4 * (trsby3 - sxy + sxz - syz);
  v[9] = rhobyb + ru + st; v[12] = rhobyb - ru + st;
  ru = dbybc2 * (rux + ruy - ruz); st = dd2bybc4 * (trsby3 + sxy - sxz - syz);
  v[10] = rhobyb - ru + st; v[11] = rhobyb + ru + st;
  for (q = 0; q < 15; q++) {
    if (average) t[q] += 0.5 * v[q];
    else t[q] = v[q];
  }
}

/* reference src/lbstore.c:36-91 */
void lbsave(LBSys lb, char *savefile) {
  long x;
  FILE *fp;
  if ((fp = fopen(savefile, "wb")) == NULL) { printf("savefile: %s could not be opened\n", savefile); return; }
  printf("\nSaving density, momentum, stress to %s\n", savefile);
  bbl(lb); propagate(lb);
  lbpull(lb);
  for (x = 0; x < lb->nnodes; x++) {
    LBStoreReal m[10];
    store_moments(lb->a + 15 * x, m);
    fwrite(m, sizeof(LBStoreReal), 10, fp);
  }
  fclose(fp);
  collide(lb);
  slb_trace(lb, "lbsave");
}

/* reference src/lbstore.c:104-218 */
void lbload(LBSys lb, char *loadfile) {
  long x;
  int q;
  FILE *fp;
  LBReal *a;
  if (lb->changed_objects) syncobjs(lb);
  if ((fp = fopen(loadfile, "r")) == NULL) { printf("lbload: %s could not be opened\n", loadfile); exit(EXIT_FAILURE); }
  printf(lb->load_average ? "\nAveraging density, momentum, stress with %s\n" : "\nLoading density, momentum, stress from %s\n", loadfile);
  if (lb->rescale != 1.0) {
    printf("Multiplying velocity field (only) by %f\n", lb->rescale);
    printf("*** this factor will be reset to unity at end of loading ***\n");
  }
  if (lb->load_average) lbpull(lb);
  a = slb_host_a(lb);
  for (x = 0; x < lb->nnodes; x++) {
    LBStoreReal s[10];
    LBStoreReal rux, ruy, ruz;
    if (fread(s, sizeof(LBStoreReal), 10, fp) != 10) memset(s, 0, sizeof s);
    rux = (lb->rescale) * s[1]; ruy = (lb->rescale) * s[2]; ruz = (lb->rescale) * s[3];
    rebuild_store(a + 15 * x, s[0], rux, ruy, ruz, s[4], s[5], s[6], s[7], s[8], s[9], lb->load_average);
  }
  fclose(fp);
  if (lb->skip_solid)
    for (x = 0; x < lb->nnodes; x++)
      if (lb->obj[x] != NULL) for (q = 0; q < 15; q++) a[q + 15 * x] = 0.0;
  slb_mark_pops(lb);
  lb->status = POST_PROPAGATE;
  collide(lb);
  lb->rescale = 1.0;
  slb_trace(lb, "lbload");
}

/* reference src/lbstore.c:227-296.  The velocity correction uses the node
 * force arrays fx, fy, fz, exactly as the reference does. */
void lbsavevel(LBSys lb, char *savefile, char *type) {
  int i, j, k, binary = (type[0] == 'b' || type[0] == 'B');
  LBReal fac = 0.0, rho = 0.0, ux, uy, uz;
  FILE *fp;
  if ((fp = fopen(savefile, "w")) == NULL) { printf("savefile: %s could not be opened\n", savefile); return; }
  if (lb->vel_corrected) {
    printf("\nSaving corrected velocity field in %s to %s", binary ? "binary" : "ascii", savefile);
    switch (lb->status) {
      case POST_BBL: printf(" [post-bounceback - not a good idea]\n"); break;
      case POST_PROPAGATE: fac = 0.5; printf("\n"); break;
      case POST_COLLIDE: fac = -0.5; printf("\n"); break;
    }
  } else {
    printf("\nSaving ");
    switch (lb->status) {
      case POST_BBL: printf("post-bounceback [not a good idea]"); break;
      case POST_PROPAGATE: printf("post-propagation"); break;
      case POST_COLLIDE: printf("post-collision"); break;
    }
    printf(" uncorrected velocity field in %s to %s\n", binary ? "binary" : "ascii", savefile);
  }
  lbpull(lb);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long x = slb_node(lb, i, j, k);
    if (lb->obj[x] != NULL && lb->skip_solid) {
      ux = uy = uz = 0.0;
    } else {
      const LBReal *t = lb->a + 15 * x;
      rho = lb->rho0 + t[0] + t[1] + t[2] + t[3] + t[4] + t[5] + t[6] + t[7] + t[8] + t[9] + t[10] + t[11] + t[12] + t[13] + t[14];
      ux = (t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14] + fac * lb->fx[x]) / rho;
      uy = (t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14] + fac * lb->fy[x]) / rho;
      uz = (t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14] + fac * lb->fz[x]) / rho;
    }
    if (binary) {
      fwrite(&rho, sizeof(LBReal), 1, fp); fwrite(&ux, sizeof(LBReal), 1, fp);
      fwrite(&uy, sizeof(LBReal), 1, fp); fwrite(&uz, sizeof(LBReal), 1, fp);
    } else {
      fprintf(fp, "%g %g %g %g %i %i %i\n", rho, ux, uy, uz, i, j, k);
    }
  }
  fclose(fp);
  slb_trace(lb, "lbsavevel");
}

/* appended: the warm start of lbloadvel from arrays (rho may be NULL, then
 * rho = rho0): reference src/lbstore.c:340-401 with the populations rebuilt
 * on the GPU, then a collision. */
void lbsetvel(LBSys lb, LBReal *rho, LBReal *ux, LBReal *uy, LBReal *uz) {
  long x, n = lb->nnodes;
  LBReal *vx, *vy, *vz;
  if (lb->changed_objects) syncobjs(lb);
  vx = (LBReal *)malloc(n * sizeof(LBReal)); vy = (LBReal *)malloc(n * sizeof(LBReal));
  vz = (LBReal *)malloc(n * sizeof(LBReal));
  if (vx == NULL || vy == NULL || vz == NULL) error("No room for velocity field");
  for (x = 0; x < n; x++) { vx[x] = lb->rescale * ux[x]; vy[x] = lb->rescale * uy[x]; vz[x] = lb->rescale * uz[x]; }
  slb_check(slbc_set_velocity(slb_device(lb), rho, vx, vy, vz, lb->skip_solid), "velocity warm start");
  free(vx); free(vy); free(vz);
  slb_device_changed(lb);
  lb->status = POST_PROPAGATE;
  collide(lb);
  lb->rescale = 1.0;
}

/* appended: lbsetvel from three device FP32 arrays (rho = rho0), so a
 * velocity field computed on the GPU never crosses to the host */
void lbsetveldev(LBSys lb, void *u) {
  if (lb->changed_objects) syncobjs(lb);
  if (lb->rescale != 1.0) printf("lbsetveldev: lb->rescale ignored (velocities used as given)\n");
  slb_check(slbc_set_velocity_dev(slb_device(lb), (const float *)u, lb->skip_solid), "velocity warm start");
  slb_device_changed(lb);
  lb->status = POST_PROPAGATE;
  collide(lb);
  lb->rescale = 1.0;
}

/* appended: the velocity field into three device FP32 arrays, with the
 * half-force correction accvmean applies when lb->vel_corrected, and with
 * lbstate the density deviation of every fluid node */
void lbstate(LBSys lb, void *u, void *drho) {
  double fac = 0.0;
  if (lb->vel_corrected) fac = lb->status == POST_PROPAGATE ? 0.5 : -0.5;
  if (lb->changed_objects) syncobjs(lb);
  slb_check(slbc_get_state_dev(slb_device(lb), fac, (float *)u, (float *)drho), "velocity field");
}

void lbvelocity(LBSys lb, void *u) { lbstate(lb, u, NULL); }

/* appended: lbsetveldev with a device field of density deviations */
void lbsetstatedev(LBSys lb, void *u, void *drho) {
  if (lb->changed_objects) syncobjs(lb);
  if (lb->rescale != 1.0) printf("lbsetstatedev: lb->rescale ignored (velocities used as given)\n");
  slb_check(slbc_set_state_dev(slb_device(lb), (const float *)u, (const float *)drho, lb->skip_solid),
            "state warm start");
  slb_device_changed(lb);
  lb->status = POST_PROPAGATE;
  collide(lb);
  lb->rescale = 1.0;
}

/* reference src/lbstore.c:305-404 */
void lbloadvel(LBSys lb, char *loadfile, char *type) {
  long x, n = lb->nnodes;
  int binary = (type[0] == 'b' || type[0] == 'B'), i, j, k;
  LBReal *r, *vx, *vy, *vz;
  FILE *fp;
  if (lb->changed_objects) syncobjs(lb);
  if (myscmp("null", loadfile)) { printf("\nNo load file\n"); return; }
  printf("\nLoading velocity field from %s file %s\n", binary ? "binary" : "ascii", loadfile);
  printf(" (approximate LB initialisation)\n");
  if ((fp = fopen(loadfile, "r")) == NULL) { printf("lbloadvel: %s could not be opened\n", loadfile); exit(EXIT_FAILURE); }
  if (lb->rescale != 1.0) {
    printf("Multiplying velocity field by %f\n", lb->rescale);
    printf("*** this factor will be reset to unity at end of loading ***\n");
  }
  r = (LBReal *)calloc(n, sizeof(LBReal)); vx = (LBReal *)calloc(n, sizeof(LBReal));
  vy = (LBReal *)calloc(n, sizeof(LBReal)); vz = (LBReal *)calloc(n, sizeof(LBReal));
  if (r == NULL || vx == NULL || vy == NULL || vz == NULL) error("No room for velocity field");
  for (x = 0; x < n; x++) {
    if (binary) {
      if (fread(&r[x], sizeof(LBReal), 1, fp) != 1 || fread(&vx[x], sizeof(LBReal), 1, fp) != 1 ||
          fread(&vy[x], sizeof(LBReal), 1, fp) != 1 || fread(&vz[x], sizeof(LBReal), 1, fp) != 1) break;
    } else {
      float tr, tx, ty, tz;
      if (fscanf(fp, "%f%f%f%f%i%i%i", &tr, &tx, &ty, &tz, &i, &j, &k) != 7) break;
      r[x] = tr; vx[x] = tx; vy[x] = ty; vz[x] = tz;
    }
  }
  fclose(fp);
  lbsetvel(lb, r, vx, vy, vz);
  free(r); free(vx); free(vy); free(vz);
  slb_trace(lb, "lbloadvel");
}

/* reference src/lbstore.c:412-515 */
void lbsavestr(LBSys lb, char *savefile, char *type) {
  long x, n = lb->nnodes;
  int c, binary = (type[0] == 'b' || type[0] == 'B');
  LBReal *s = (LBReal *)calloc(6 * (size_t)n, sizeof(LBReal));
  FILE *fp;
  if (s == NULL) { printf("lbsavestr: ran out of memory for temporary storage\n"); return; }
  bbl(lb); propagate(lb);
  lbpull(lb);
  for (x = 0; x < n; x++) {
    LBReal m[10];
    moments(lb->a + 15 * x, m);
    for (c = 0; c < 6; c++) s[6 * x + c] = m[4 + c];
  }
  collide(lb);
  lbpull(lb);
  for (x = 0; x < n; x++) {
    LBReal m[10];
    moments(lb->a + 15 * x, m);
    for (c = 0; c < 6; c++) s[6 * x + c] += m[4 + c];
  }
  if ((fp = fopen(savefile, "wb")) == NULL) { printf("savefile: %s could not be opened\n", savefile); free(s); return; }
  printf("\nSaving stress field in %s to %s\n", binary ? "binary" : "ascii", savefile);
  for (x = 0; x < n; x++) {
    LBReal t[6];
    int void_space = lb->obj[x] == NULL;
    for (c = 0; c < 6; c++) t[c] = (!void_space && lb->skip_solid) ? 0.0 : 0.5 * s[6 * x + c];
    if (binary) {
      for (c = 0; c < 6; c++) fwrite(&t[c], sizeof(LBStoreReal), 1, fp);
      fwrite(&void_space, sizeof(int), 1, fp);
    } else {
      fprintf(fp, "%f\t%f\t%f\t%f\t%f\t%f\t%i\n", t[0], t[1], t[2], t[3], t[4], t[5], void_space);
    }
  }
  fclose(fp);
  free(s);
  slb_trace(lb, "lbsavestr");
}

/* reference src/lbstore.c:523-545 */
void lbsaveobj(LBSys lb, char *savefile) {
  int more = 0;
  FILE *fp;
  LBObj p;
  if (myscmp("stdout", savefile)) { fp = stdout; more = 1; }
  else if (myscmp("stderr", savefile)) { fp = stderr; more = 1; }
  else if ((fp = fopen(savefile, "w")) == NULL) { printf("lbsaveobj: %s could not be opened\n", savefile); return; }
  printf("\nSaving object data to %s\n", savefile);
  if (more) fprintf(fp, "START of particle data: TYPE, id, base id, x, y, z\n\n");
  for (p = lb->obj_head; p != NULL; p = p->next_obj) {
    fprintf(fp, "POS %3i %3i %f %f %f\n", p->id, p->base_obj->id, p->posx, p->posy, p->posz);
    fprintf(fp, "VEL %3i %3i %f %f %f\n", p->id, p->base_obj->id, p->velx, p->vely, p->velz);
    fprintf(fp, "ANG %3i %3i %f %f %f\n", p->id, p->base_obj->id, p->angx, p->angy, p->angz);
    fprintf(fp, "FRC %3i %3i %f %f %f\n", p->id, p->base_obj->id, p->frcx, p->frcy, p->frcz);
    fprintf(fp, "TRQ %3i %3i %f %f %f\n", p->id, p->base_obj->id, p->trqx, p->trqy, p->trqz);
    if (more) fprintf(fp, "\n");
  }
  if (more) fprintf(fp, "END of particle data\n");
  if (fp != stdout && fp != stderr) fclose(fp);
  slb_trace(lb, "lbsaveobj");
}

/* reference src/lbstore.c:554-586 */
void lbloadobj(LBSys lb, char *loadfile) {
  int irc = 0, i1, i2;
  float t1, t2, t3;
  FILE *fp;
  LBObj p1;
  if ((fp = fopen(loadfile, "r")) == NULL) { printf("lbloadobj: %s could not be opened\n", loadfile); return; }
  printf("Loading object data from %s\n", loadfile);
  if (lb->rescale != 1.0) {
    printf("Multiplying velocities and angular velocities by %f\n", lb->rescale);
    printf("*** this factor will be reset to unity at end of loading ***\n");
  }
  while (fscanf(fp, "%*s%i%i%f%f%f", &i1, &i2, &t1, &t2, &t3) == 5) {
    if ((p1 = lookupobj(lb, i1)) == NULL) { irc = 1; break; }
    if (i2 != i1) {
      if (lookupobj(lb, i2) == NULL) { irc = 2; break; }
      p1->base_obj->id = i2;
    }
    p1->posx = t1; p1->posy = t2; p1->posz = t3;
    if (fscanf(fp, "%*s%i%i%f%f%f", &i1, &i2, &t1, &t2, &t3) != 5) { irc = 3; break; }
    p1->velx = lb->rescale * t1; p1->vely = lb->rescale * t2; p1->velz = lb->rescale * t3;
    if (fscanf(fp, "%*s%i%i%f%f%f", &i1, &i2, &t1, &t2, &t3) != 5) { irc = 4; break; }
    p1->angx = lb->rescale * t1; p1->angy = lb->rescale * t2; p1->angz = lb->rescale * t3;
    if (fscanf(fp, "%*s%i%i%f%f%f", &i1, &i2, &t1, &t2, &t3) != 5) { irc = 5; break; }
    if (fscanf(fp, "%*s%i%i%f%f%f", &i1, &i2, &t1, &t2, &t3) != 5) { irc = 6; break; }
  }
  if (irc == 1 || irc == 2) printf("UFO found (unidentified floating object)\n");
  if (irc > 3) printf("Ran out of data apparently\n");
  fclose(fp);
  lb->rescale = 1.0;
  slb_trace(lb, "lbloadobj");
}

/* reference src/lbstore.c:595-640 */
void lbsavefrc(LBSys lb, char *frcfile, char *type) {
  int i, j, k, binary = (type[0] == 'b' || type[0] == 'B'), list = (type[0] == 'l' || type[0] == 'L');
  FILE *fp;
  if ((fp = fopen(frcfile, "w")) == NULL) { printf("lbsavefrc: %s could not be opened\n", frcfile); exit(EXIT_FAILURE); }
  lbpull(lb);
  if (list) {
    printf("\nSaving force data as a list to %s\n", frcfile);
    for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
      long x = slb_node(lb, i, j, k);
      if (lb->mask[x] > 0) {
        LBObj p = lb->obj[x];
        fprintf(fp, "%i %i %i %f %f %f %i %f %f %f\n", i, j, k, lb->fx[x], lb->fy[x], lb->fz[x],
                p->id, p->posx, p->posy, p->posz);
      }
    }
  } else {
    long x;
    printf("\nSaving %s force data to %s\n", binary ? "binary" : "ascii", frcfile);
    for (x = 0; x < lb->nnodes; x++) {
      LBStoreReal f[3];
      f[0] = lb->fx[x]; f[1] = lb->fy[x]; f[2] = lb->fz[x];
      if (binary) fwrite(f, sizeof(LBStoreReal), 3, fp);
      else fprintf(fp, "%f %f %f\n", f[0], f[1], f[2]);
    }
  }
  fclose(fp);
  slb_trace(lb, "lbsavefrc");
}

/* reference src/lbstore.c:647-678 */
void lbsavemap(LBSys lb, char *mapfile, char *type) {
  int i, j, k;
  FILE *fp;
  if ((fp = fopen(mapfile, "w")) == NULL) { printf("lbsavemap: %s could not be opened\n", mapfile); exit(EXIT_FAILURE); }
  if (type[0] == 'l' || type[0] == 'L') {
    printf("\nSaving list of solid nodes to %s\n", mapfile);
    for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++)
      if (lb->obj[slb_node(lb, i, j, k)] != NULL) fprintf(fp, "%i %i %i\n", i, j, k);
  } else {
    long x;
    printf("\nSaving object map as character array to %s\n", mapfile);
    for (x = 0; x < lb->nnodes; x++) fputc(lb->obj[x] == NULL ? 0 : 255, fp);
  }
  fclose(fp);
  slb_trace(lb, "lbsavemap");
}

/* ---- signals: reference src/lbsignal.c ----------------------------------- */
#ifdef SIGNAL
int slb_signal_flag = 0;

void sighandle(LBSys lb) {
  if (slb_signal_flag == 0) return;
  if (slb_signal_flag == 1) {
    printf("Acting on -USR1 signal\n");
    if (lb->name != NULL) wrmon(lb, "running");
  } else if (slb_signal_flag == 2) {
    printf("Acting on -USR2 signal\n");
    if (lb->name != NULL) {
      char *dms = mycat(lb->name, ".dms"), *objf = mycat(lb->name, ".obj");
      slb_signal_flag = 0;  /* lbsave collides, which would poll again */
      lbsave(lb, dms);
      if (lb->obj_head != NULL) lbsaveobj(lb, objf);
      free(dms); free(objf);
    }
  }
  slb_signal_flag = 0;
  slb_trace(lb, "sighandle");
}

void sighook(int sig) {
  int flag = 0;
  if (sig == SIGUSR1) { flag = 1; signal(SIGUSR1, sighook); }
  else if (sig == SIGUSR2) { flag = 2; signal(SIGUSR2, sighook); }
  if (slb_signal_flag == 0) slb_signal_flag = flag;
}

void siginit() {
  slb_signal_flag = 0;
  signal(SIGUSR1, sighook);
  signal(SIGUSR2, sighook);
}
#endif
