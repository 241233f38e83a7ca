/*
 * Objects and geometry (host side of reference src/lbobjs.c): the object
 * list, shape rasterisation into the object map lb->obj, the boundary-link
 * mask, wall velocities and body force.  These are set-up routines; each
 * one records which host arrays it changed so the next device call uploads
 * them (slb_core.c).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "slb_private.h"

static const int LX[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
static const int LY[15] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const int LZ[15] = {0, 0, 0, 0, 0, 1, -1, 1, 1, 1, 1, -1, -1, -1, -1};

/* reference src/lbobjs.c:33-52 */
LBObj addobj(LBSys lb) {
  LBObj p = (LBObj)malloc(sizeof(LBObj_type));
  if (p == NULL) error("Ran out of memory for object creation\n");
  p->base_obj = p;
  p->id = lb->next_id++;
  p->next_obj = lb->obj_head;
  lb->obj_head = p;
  return p;
}

/* reference src/lbobjs.c:57-63 */
void zeroobj(LBObj p) {
  p->posx = p->posy = p->posz = 0.0;
  p->velx = p->vely = p->velz = 0.0;
  p->angx = p->angy = p->angz = 0.0;
  p->frcx = p->frcy = p->frcz = 0.0;
  p->trqx = p->trqy = p->trqz = 0.0;
}

/* reference src/lbobjs.c:68-72 */
LBObj lookupobj(LBSys lb, int tid) {
  LBObj p;
  for (p = lb->obj_head; p != NULL; p = p->next_obj)
    if (p->id == tid) return p;
  return NULL;
}

/* an insert routine that set no node drops its new object again */
static LBObj drop_new(LBSys lb, LBObj p, int undo_id) {
  if (slb_verbosity & OBJECT_DETAILS) printf("No sites set in object\n");
  lb->obj_head = p->next_obj;
  free(p);
  if (undo_id) lb->next_id--;
  return NULL;
}

static void set_node(LBSys lb, long x, LBObj p, int *ns, int *overlap) {
  if (lb->obj[x] != NULL) *overlap = 1;
  lb->obj[x] = p;
  (*ns)++;
}

static void map_changed(LBSys lb) {
  lb->changed_objects = 1;
  slb_mark_geometry(lb);
}

/* reference src/lbobjs.c:77-123 */
LBObj insertsubs(LBSys lb, char *subsfile, int ilo, int ihi, int jlo, int jhi, int klo, int khi) {
  int i, j, k, ns = 0, overlap = 0, done = 0;
  unsigned char byte;
  FILE *fp;
  LBObj p;
  if ((fp = fopen(subsfile, "r")) == NULL) {
    printf("insertsubs: %s could not be opened\n", subsfile);
    return NULL;
  }
  if (slb_verbosity & OBJECT_DETAILS) {
    printf("\nInserting substrate data from %s\n", subsfile);
    printf("Substrate region is (%i-%i, %i-%i, %i-%i) inclusive\n", ilo, ihi, jlo, jhi, klo, khi);
  }
  p = addobj(lb);
  zeroobj(p);
  for (i = ilo; i <= ihi && !done; i++)
    for (j = jlo; j <= jhi && !done; j++)
      for (k = klo; k <= khi; k++) {
        if (fscanf(fp, "%c", &byte) != 1) {
          if (slb_verbosity & OBJECT_DETAILS) printf("Ran out of data in %s\n", subsfile);
          break;
        }
        if (byte & 1) set_node(lb, slb_node(lb, i, j, k), p, &ns, &overlap);
      }
  if (slb_verbosity & OBJECT_DETAILS) {
    printf("Inserted substrate data, id no = %i, # nodes = %i\n", p->id, ns);
    if (overlap) printf("Overlaps occurred\n");
  }
  if (ns == 0) { fclose(fp); return drop_new(lb, p, 0); }
  map_changed(lb);
  fclose(fp);
  slb_trace(lb, "insertsubs");
  return p;
}

/* reference src/lbobjs.c:128-165 */
LBObj insertlist(LBSys lb, char *listfile) {
  int i, j, k, ns = 0, overlap = 0;
  FILE *fp;
  LBObj p;
  if ((fp = fopen(listfile, "r")) == NULL) {
    printf("insertlist: %s could not be opened\n", listfile);
    return NULL;
  }
  if (slb_verbosity & OBJECT_DETAILS) printf("\nInserting substrate node list data from %s\n", listfile);
  p = addobj(lb);
  zeroobj(p);
  while (fscanf(fp, "%i%i%i", &i, &j, &k) == 3) {
    if (i >= 0 && i < lb->esi && j >= 0 && j < lb->esj && k >= 0 && k < lb->esk)
      set_node(lb, slb_node(lb, i, j, k), p, &ns, &overlap);
    else if (slb_verbosity & OBJECT_DETAILS)
      printf("insertlist: ignoring node (%i,%i,%i), it is out of range\n", i, j, k);
  }
  if (slb_verbosity & OBJECT_DETAILS) {
    printf("Inserted node list data, id no = %i, # nodes = %i\n", p->id, ns);
    if (overlap) printf("Overlaps occurred\n");
  }
  fclose(fp);
  if (ns == 0) return drop_new(lb, p, 0);
  map_changed(lb);
  slb_trace(lb, "insertlist");
  return p;
}

/* appended: one object made of the nodes where mask[inode] != 0 (the node
 * list of insertlist held in memory, inode = esk*(esj*i+j)+k) */
LBObj insertmask(LBSys lb, unsigned char *mask) {
  long x;
  int ns = 0, overlap = 0;
  LBObj p = addobj(lb);
  zeroobj(p);
  for (x = 0; x < lb->nnodes; x++)
    if (mask[x]) set_node(lb, x, p, &ns, &overlap);
  if (slb_verbosity & OBJECT_DETAILS) {
    printf("Inserted node mask, id no = %i, # nodes = %i\n", p->id, ns);
    if (overlap) printf("Overlaps occurred\n");
  }
  if (ns == 0) return drop_new(lb, p, 0);
  map_changed(lb);
  slb_trace(lb, "insertmask");
  return p;
}

/* reference src/lbobjs.c:170-199 */
LBObj insertslab(LBSys lb, LBReal x1, LBReal x2, LBReal y1, LBReal y2, LBReal z1, LBReal z2) {
  int i, j, k, ns = 0, overlap = 0;
  LBObj p = addobj(lb);
  zeroobj(p);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++)
    if (i > x1 && i < x2 && j > y1 && j < y2 && k > z1 && k < z2)
      set_node(lb, slb_node(lb, i, j, k), p, &ns, &overlap);
  if (slb_verbosity & OBJECT_DETAILS) {
    printf("Inserted slab %5.2f < x < %5.2f, %5.2f < y < %5.2f, %5.2f < z < %5.2f, ", x1, x2, y1, y2, z1, z2);
    printf("   id no = %i, # nodes = %i\n", p->id, ns);
    if (overlap) printf("Overlaps occurred\n");
  }
  if (ns == 0) return drop_new(lb, p, 0);
  map_changed(lb);
  p->posx = 0.5 * (x1 + x2 - 1); p->posy = 0.5 * (y1 + y2 - 1); p->posz = 0.5 * (z1 + z2 - 1);
  slb_trace(lb, "insertslab");
  return p;
}

/* index range [*lo, *hi] that holds every node within rad of c (one node of
 * margin; the exact test below decides membership) */
static void bound(LBReal c, LBReal rad, int n, int *lo, int *hi) {
  double a = floor(c - rad) - 1.0, b = ceil(c + rad) + 1.0;
  *lo = a < 0.0 ? 0 : (a > n - 1 ? n : (int)a);
  *hi = b > n - 1 ? n - 1 : (b < 0.0 ? -1 : (int)b);
}

/* reference src/lbobjs.c:204-232.  Only the bounding box of the sphere is
 * scanned; the membership test rsq < radsq is the reference's, so the node
 * set, node count and overlap flag are identical. */
LBObj insertsph(LBSys lb, LBReal rad, LBReal ox, LBReal oy, LBReal oz) {
  int i, j, k, ns = 0, overlap = 0;
  int i0 = 0, i1 = lb->esi - 1, j0 = 0, j1 = lb->esj - 1, k0 = 0, k1 = lb->esk - 1;
  LBReal rsq, radsq = rad * rad;
  LBObj p = addobj(lb);
  zeroobj(p);
  if (isfinite(rad) && isfinite(ox) && isfinite(oy) && isfinite(oz)) {
    LBReal r = fabs(rad);
    bound(ox, r, lb->esi, &i0, &i1);
    bound(oy, r, lb->esj, &j0, &j1);
    bound(oz, r, lb->esk, &k0, &k1);
  }
  for (i = i0; i <= i1; i++) for (j = j0; j <= j1; j++) for (k = k0; k <= k1; k++) {
    rsq = (i - ox) * (i - ox) + (j - oy) * (j - oy) + (k - oz) * (k - oz);
    if (rsq < radsq) set_node(lb, slb_node(lb, i, j, k), p, &ns, &overlap);
  }
  if (slb_verbosity & OBJECT_DETAILS) {
    printf("Sphere radius %5.2f at %6.2f %6.2f %6.2f ", rad, ox, oy, oz);
    printf("id = %5i, # nodes = %i", p->id, ns);
    printf(overlap ? " (overlaps)\n" : "\n");
  }
  if (ns == 0) return drop_new(lb, p, 1);
  map_changed(lb);
  p->posx = ox; p->posy = oy; p->posz = oz;
  slb_trace(lb, "insertsph");
  return p;
}

/* appended: n insertsph calls (reference src/lbobjs.c:204-232) at once, the
 * node tests done on the GPU: the same objects (one per sphere that covers
 * a node, ids in order, pos = centre), the same map (a later sphere takes a
 * node over from an earlier one) and the same messages.  Returns the number
 * of objects created. */
int insertspheres(LBSys lb, int n, LBReal *rad, LBReal *ox, LBReal *oy, LBReal *oz) {
  long x, nn = lb->nnodes;
  int s, made = 0;
  double *sph;
  int *last, *count;
  unsigned char *taken, *overlap;
  LBObj *objs;
  if (n <= 0) return 0;
  sph = (double *)malloc((size_t)n * 4 * sizeof(double));
  count = (int *)calloc((size_t)n, sizeof(int));
  overlap = (unsigned char *)calloc((size_t)n, 1);
  objs = (LBObj *)calloc((size_t)n, sizeof(LBObj));
  last = (int *)malloc((size_t)nn * sizeof(int));
  taken = (unsigned char *)malloc((size_t)nn);
  if (!sph || !count || !overlap || !objs || !last || !taken) error("No room for the sphere list");
  for (s = 0; s < n; s++) {
    sph[4 * s] = rad[s]; sph[4 * s + 1] = ox[s]; sph[4 * s + 2] = oy[s]; sph[4 * s + 3] = oz[s];
  }
  for (x = 0; x < nn; x++) taken[x] = lb->obj[x] != NULL;
  slb_check(slbc_raster_spheres(lb->esi, lb->esj, lb->esk, n, sph, taken, last, count, overlap),
            "sphere rasterisation");
  for (s = 0; s < n; s++) {
    LBObj p = addobj(lb);
    zeroobj(p);
    if (slb_verbosity & OBJECT_DETAILS) {
      printf("Sphere radius %5.2f at %6.2f %6.2f %6.2f ", rad[s], ox[s], oy[s], oz[s]);
      printf("id = %5i, # nodes = %i", p->id, count[s]);
      printf(overlap[s] ? " (overlaps)\n" : "\n");
    }
    if (count[s] == 0) { drop_new(lb, p, 1); continue; }
    p->posx = ox[s]; p->posy = oy[s]; p->posz = oz[s];
    objs[s] = p;
    made++;
  }
  for (x = 0; x < nn; x++)
    if (last[x] >= 0) lb->obj[x] = objs[last[x]];
  if (made) map_changed(lb);
  free(sph); free(count); free(overlap); free(objs); free(last); free(taken);
  slb_trace(lb, "insertspheres");
  return made;
}

/* reference src/lbobjs.c:241-287 */
LBObj insertcyl(LBSys lb, char *type, LBReal rad, LBReal a, LBReal b) {
  int i, j, k, ns = 0, overlap = 0, within;
  LBReal rsq = 0.0, radsq = rad * rad;
  LBObj p = addobj(lb);
  zeroobj(p);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    switch (type[0]) {
      case 'x': case 'i': rsq = (j - a) * (j - a) + (k - b) * (k - b); break;
      case 'y': case 'j': rsq = (i - a) * (i - a) + (k - b) * (k - b); break;
      case 'z': case 'k': rsq = (i - a) * (i - a) + (j - b) * (j - b); break;
      default: error("Unrecognised cylinder direction"); return NULL;
    }
    within = (rsq < radsq);
    if (type[1] != '\0') within = !within;
    if (within) set_node(lb, slb_node(lb, i, j, k), p, &ns, &overlap);
  }
  if (slb_verbosity & OBJECT_DETAILS) {
    printf(type[1] == '\0' ? "Cylinder " : "Cylindrical hole ");
    printf("radius %5.2f, axis %5.2f %5.2f along %c ", rad, a, b, type[0]);
    printf("id = %i, # nodes = %i", p->id, ns);
    if (ns == 0) printf(" (no sites set)");
    printf(overlap ? " (overlaps)\n" : "\n");
  }
  if (ns == 0) {
    lb->obj_head = p->next_obj; free(p); lb->next_id--;
    return NULL;
  }
  map_changed(lb);
  switch (type[0]) {
    case 'x': case 'i': p->posx = 0.5 * (lb->esi - 1); p->posy = a; p->posz = b; break;
    case 'y': case 'j': p->posx = a; p->posy = 0.5 * (lb->esj - 1); p->posz = b; break;
    default: p->posx = a; p->posy = b; p->posz = 0.5 * (lb->esk - 1); break;
  }
  slb_trace(lb, "insertcyl");
  return p;
}

/* reference src/lbobjs.c:294-357.  As in the reference, a bad direction or
 * an out-of-range position returns NULL and leaves the new, empty object in
 * the list. */
LBObj insertwall(LBSys lb, char *type, int wallpos) {
  int i, j, k, ns = 0, overlap = 0, axis, lim;
  LBObj p = addobj(lb);
  zeroobj(p);
  switch (type[0]) {
    case 'x': case 'i': axis = 0; lim = lb->esi; break;
    case 'y': case 'j': axis = 1; lim = lb->esj; break;
    case 'z': case 'k': axis = 2; lim = lb->esk; break;
    default: printf("insertwall: unrecognised direction for walls\n"); return NULL;
  }
  if (wallpos < 0 || wallpos > lim - 1) { printf("insertwall: wallpos out of range\n"); return NULL; }
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    int c = axis == 0 ? i : axis == 1 ? j : k;
    if (c == wallpos) set_node(lb, slb_node(lb, i, j, k), p, &ns, &overlap);
  }
  p->posx = axis == 0 ? wallpos : 0.5 * (lb->esi - 1);
  p->posy = axis == 1 ? wallpos : 0.5 * (lb->esj - 1);
  p->posz = axis == 2 ? wallpos : 0.5 * (lb->esk - 1);
  if (ns == 0) return drop_new(lb, p, 0);
  map_changed(lb);
  if (slb_verbosity & OBJECT_DETAILS) {
    printf("Inserted wall at %c = %i, id no = %i, # nodes = %i\n", type[0], wallpos, p->id, ns);
    if (overlap) printf("Overlaps occurred\n");
  }
  slb_trace(lb, "insertwall");
  return p;
}

static void free_objects(LBSys lb) {
  LBObj p = lb->obj_head, pp;
  while (p != NULL) { pp = p; p = p->next_obj; free(pp); }
  lb->next_id = 0;
  lb->obj_head = NULL;
}

/* reference src/lbobjs.c:362-392 (invert = 0) and 397-428 (invert = 1) */
static LBObj merge(LBSys lb, int invert) {
  int i, j, k, ns = 0;
  LBReal ox = 0.0, oy = 0.0, oz = 0.0;
  LBObj p;
  free_objects(lb);
  p = addobj(lb);
  zeroobj(p);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long x = slb_node(lb, i, j, k);
    if (invert) {
      if (lb->obj[x] != NULL) { lb->obj[x] = NULL; continue; }
    } else if (lb->obj[x] == NULL) continue;
    ox += (double)i; oy += (double)j; oz += (double)k; ns++;
    lb->obj[x] = p;
  }
  slb_mark_geometry(lb);
  if (ns == 0) return drop_new(lb, p, 0);
  lb->changed_objects = 1;
  if (slb_verbosity & OBJECT_DETAILS)
    printf("Object space %s to id no %i, # nodes = %i\n", invert ? "inverted" : "flattened", p->id, ns);
  p->posx = ox / ns; p->posy = oy / ns; p->posz = oz / ns;
  slb_trace(lb, invert ? "invertobj" : "flattenobj");
  return p;
}
LBObj flattenobj(LBSys lb) { return merge(lb, 0); }
LBObj invertobj(LBSys lb) { return merge(lb, 1); }

/* reference src/lbobjs.c:433-453: no objects, wall velocity, node force
 * and populations all zero. */
void removeobjs(LBSys lb) {
  long x;
  free_objects(lb);
  for (x = 0; x < lb->nnodes; x++) {
    lb->obj[x] = NULL;
    lb->ux[x] = lb->uy[x] = lb->uz[x] = 0.0;
    lb->fx[x] = lb->fy[x] = lb->fz[x] = 0.0;
  }
  memset(slb_host_a(lb), 0, 15 * (size_t)lb->nnodes * sizeof(LBReal));
  slb_mark_pops(lb);
  slb_mark_wallvel(lb);
  slb_state(lb)->host_f_valid = 1;
  if (slb_verbosity & OBJECT_DETAILS) printf("All objects removed\n");
  map_changed(lb);
  slb_trace(lb, "removeobjs");
}

/* reference src/lbobjs.c:457-467 */
void wrobjs(LBSys lb) {
  LBObj p;
  for (p = lb->obj_head; p != NULL; p = p->next_obj) {
    printf("Object id (base) = %i (%i)\n", p->id, p->base_obj->id);
    printf(" posx, y, z = %f %f %f\n", p->posx, p->posy, p->posz);
    printf(" velx, y, z = %f %f %f\n", p->velx, p->vely, p->velz);
    printf(" angx, y, z = %f %f %f\n", p->angx, p->angy, p->angz);
    printf(" frcx, y, z = %f %f %f\n", p->frcx, p->frcy, p->frcz);
    printf(" trqx, y, z = %f %f %f\n", p->trqx, p->trqy, p->trqz);
  }
}

/* reference src/lbobjs.c:472-516 */
void wrmap(LBSys lb, char *name) {
  static const char shape[] = "ox+*#acemnrsuvwxz?";
  int len = (int)strlen(shape), count[32], i, j, k;
  FILE *fp = fopen(name, "w");
  if (fp == NULL) { fprintf(stderr, "Couldn't open %s\n", name); return; }
  memset(count, 0, sizeof count);
  for (k = 0; k < lb->esk; k++) {
    fprintf(fp, "\nSlice k = %3i\n            ", k);
    for (i = 0; i < lb->esi; i++) fprintf(fp, "%c", i < 10 ? ' ' : ('0' + (i / 10) % 10));
    fprintf(fp, "\nCol i =     ");
    for (i = 0; i < lb->esi; i++) fprintf(fp, "%c", '0' + (i % 10));
    fprintf(fp, "\n");
    for (j = 0; j < lb->esj; j++) {
      fprintf(fp, "Row j = %3i ", j);
      for (i = 0; i < lb->esi; i++) {
        LBObj p = lb->obj[slb_node(lb, i, j, k)];
        char c = '.';
        if (p != NULL) {
          int id = p->id >= len ? len - 1 : (p->id < 0 ? len - 1 : p->id);
          c = shape[id];
          count[id]++;
        }
        fprintf(fp, "%c", c);
      }
      fprintf(fp, "\n");
    }
  }
  fclose(fp);
  printf("\n id shape count\n");
  for (i = 0; i < len; i++) if (count[i] > 0) printf("%3i   %c %6i\n", i, shape[i], count[i]);
  printf("\nMap of object space written to %s\n", name);
}

/* reference src/lbobjs.c:526-560: bit q-1 of the mask of a solid node is set
 * when its neighbour along link q is fluid; fluid nodes get 0 (which also
 * clears any adsorption bit, as in the reference). */
void makemask(LBSys lb) {
  int i, j, k, q;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long x = slb_node(lb, i, j, k);
    int val = 0;
    if (lb->obj[x] != NULL)
      for (q = 1; q < 15; q++) {
        int ii = (i + LX[q] + lb->esi) % lb->esi;
        int jj = (j + LY[q] + lb->esj) % lb->esj;
        int kk = (k + LZ[q] + lb->esk) % lb->esk;
        if (lb->obj[slb_node(lb, ii, jj, kk)] == NULL) val |= 1 << (q - 1);
      }
    lb->mask[x] = val;
  }
  slb_mark_ads(lb);
  slb_trace(lb, "makemask");
}

/* wall velocity times rho0/12 of object p at node (i,j,k):
 * reference src/lbobjs.c:582-585 */
static void wall_u(LBSys lb, LBObj p, int i, int j, int k, LBReal *u) {
  LBReal rx = i - p->posx, ry = j - p->posy, rz = k - p->posz, rho0 = lb->rho0;
  u[0] = rho0 * ((p->velx) + (p->angy) * rz - (p->angz) * ry) / 12.0;
  u[1] = rho0 * ((p->vely) + (p->angz) * rx - (p->angx) * rz) / 12.0;
  u[2] = rho0 * ((p->velz) + (p->angx) * ry - (p->angy) * rx) / 12.0;
}

/* reference src/lbobjs.c:565-589 */
void vspread(LBSys lb) {
  int i, j, k;
  LBReal u[3];
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long x = slb_node(lb, i, j, k);
    LBObj p = lb->obj[x];
    if (p == NULL) { lb->ux[x] = lb->uy[x] = lb->uz[x] = 0.0; continue; }
    wall_u(lb, p, i, j, k, u);
    lb->ux[x] = u[0]; lb->uy[x] = u[1]; lb->uz[x] = u[2];
  }
  slb_mark_wallvel(lb);
  slb_trace(lb, "vspread");
}

/* mask bits of one node (reference src/lbobjs.c:537-556): bit q-1 when the
 * node is solid and its neighbour along c_q is fluid; clears 0x4000 */
static void mask_node(LBSys lb, int i, int j, int k) {
  long x = slb_node(lb, i, j, k);
  int q, val = 0;
  if (lb->obj[x] != NULL)
    for (q = 1; q < 15; q++) {
      int ii = (i + LX[q] + lb->esi) % lb->esi;
      int jj = (j + LY[q] + lb->esj) % lb->esj;
      int kk = (k + LZ[q] + lb->esk) % lb->esk;
      if (lb->obj[slb_node(lb, ii, jj, kk)] == NULL) val |= 1 << (q - 1);
    }
  lb->mask[x] = val;
}

/* appended, no counterpart in the reference (which can only remove objects
 * and insert new ones): move the spherical object p of radius rad -- a
 * sphere and its periodic images, as insertsph and flattenobj build it --
 * so that its centre is (x, y, z).  The node set is re-rasterised on the
 * GPU; nodes the sphere leaves become fluid at the equilibrium of density
 * rho0 and the wall velocity there (v + w x r, r = node - new centre),
 * fluid nodes it reaches join the object with their populations as they
 * are; nodes of other objects are left alone.  The host copies follow:
 * object map, mask (adsorption bits of the changed nodes and their
 * neighbours cleared), fluid count, a uniform body force (given to the new
 * fluid nodes and taken from the new solid ones; a per-node force is left
 * as it is), the wall velocities of the object when objects move, and
 * p->pos.  FP32 or FP64 populations. */
void lbtranslate(LBSys lb, LBObj p, LBReal rad, LBReal x, LBReal y, LBReal z) {
  slb_priv *st;
  slbc_lattice *dev;
  int oi = -1, e, uniform, ads_touched = 0, a;
  double oldc[3], newc[3], vel[3], ang[3], b[3];
  long cap, nch = 0, nb = 0, box = 1;
  int *changed;
  if (p == NULL) { printf("lbtranslate: no object\n"); return; }
  if (lb->changed_objects) syncobjs(lb);
  dev = slb_device(lb);
  st = slb_state(lb);
  for (e = 0; e < st->nobj; e++) if (st->objs[e] == p) { oi = e; break; }
  if (oi < 0) { printf("lbtranslate: object %i has no nodes on the lattice\n", p->id); return; }
  oldc[0] = p->posx; oldc[1] = p->posy; oldc[2] = p->posz;
  newc[0] = x; newc[1] = y; newc[2] = z;
  vel[0] = p->velx; vel[1] = p->vely; vel[2] = p->velz;
  ang[0] = p->angx; ang[1] = p->angy; ang[2] = p->angz;
  {
    int dims[3] = {lb->esi, lb->esj, lb->esk};
    for (a = 0; a < 3; a++) {
      double span = fabs(newc[a] - oldc[a]) + 2.0 * rad + 4.0;
      box *= span < dims[a] ? (long)span : dims[a];
    }
  }
  cap = box;
  changed = (int *)calloc(2 * (size_t)cap, sizeof(int));
  if (changed == NULL) error("No room for the changed-node list");
  uniform = slbc_bodyforce_uniform(dev, b);
  free(st->bnd_node); free(st->bnd_obj);
  st->bnd_node = NULL; st->bnd_obj = NULL;
  slb_check(slbc_move_sphere(dev, oi, rad, oldc, newc, vel, ang, lb->objects_moving && st->uw_sent == st->uw_gen,
                             changed, cap, &nch, st->nobj, st->objidx, &st->bnd_node, &st->bnd_obj, &nb),
            "sphere translation");
  st->nbnd = nb;
  p->posx = x; p->posy = y; p->posz = z;
  for (e = 0; e < nch; e++) {
    long n = changed[2 * e];
    int now_solid = changed[2 * e + 1] >= 0;
    lb->obj[n] = now_solid ? p : NULL;
    st->nfluid += now_solid ? -1 : 1;
    if (uniform) {
      lb->bx[n] = now_solid ? 0.0 : b[0];
      lb->by[n] = now_solid ? 0.0 : b[1];
      lb->bz[n] = now_solid ? 0.0 : b[2];
    }
    if (lb->objects_moving && !now_solid) lb->ux[n] = lb->uy[n] = lb->uz[n] = 0.0;
  }
  /* mask of the changed nodes and of their neighbours */
  for (e = 0; e < nch; e++) {
    long n = changed[2 * e];
    int k = (int)(n % lb->esk), j = (int)((n / lb->esk) % lb->esj), i = (int)(n / ((long)lb->esk * lb->esj)), q;
    for (q = 0; q < 15; q++) {
      int ii = (i + LX[q] + lb->esi) % lb->esi, jj = (j + LY[q] + lb->esj) % lb->esj;
      int kk = (k + LZ[q] + lb->esk) % lb->esk;
      long m = slb_node(lb, ii, jj, kk);
      if (lb->mask[m] & 0x4000) ads_touched = 1;  /* adsorption bit, cleared by the rebuild */
      mask_node(lb, ii, jj, kk);
    }
  }
  /* wall velocities of the object's nodes around the sphere (vspread) */
  if (lb->objects_moving) {
    int lo[3], len[3], dims[3] = {lb->esi, lb->esj, lb->esk}, ia, ib, ic;
    LBReal u[3];
    for (a = 0; a < 3; a++) {
      double l0 = floor(newc[a] - rad - 1.0), l1 = ceil(newc[a] + rad + 1.0);
      lo[a] = (int)l0;
      len[a] = (int)(l1 - l0) + 1;
      if (len[a] >= dims[a]) { lo[a] = 0; len[a] = dims[a]; }
    }
    for (ia = 0; ia < len[0]; ia++) for (ib = 0; ib < len[1]; ib++) for (ic = 0; ic < len[2]; ic++) {
      int i = ((lo[0] + ia) % dims[0] + dims[0]) % dims[0];
      int j = ((lo[1] + ib) % dims[1] + dims[1]) % dims[1];
      int k = ((lo[2] + ic) % dims[2] + dims[2]) % dims[2];
      long n = slb_node(lb, i, j, k);
      if (lb->obj[n] != p) continue;
      wall_u(lb, p, i, j, k, u);
      lb->ux[n] = u[0]; lb->uy[n] = u[1]; lb->uz[n] = u[2];
    }
    if (st->uw_sent != st->uw_gen) slb_mark_wallvel(lb);  /* not on the GPU yet: full upload */
  }
  free(changed);
  if (ads_touched) slb_mark_ads(lb);
  st->host_f_valid = 0;
  lb->changed_objects = 0;
  slb_trace(lb, "lbtranslate");
}

/* reference src/lbobjs.c:593-604 */
void zerobf(LBSys lb) {
  long x;
  for (x = 0; x < lb->nnodes; x++)
    if (lb->obj[x] == NULL) lb->bx[x] = lb->by[x] = lb->bz[x] = 0.0;
  slb_mark_bodyforce(lb);
  slb_trace(lb, "zerobf");
}

/* reference src/lbobjs.c:608-619 */
void addbf(LBSys lb, double dpdx, double dpdy, double dpdz) {
  long x;
  for (x = 0; x < lb->nnodes; x++)
    if (lb->obj[x] == NULL) {
      lb->bx[x] += (LBReal)dpdx; lb->by[x] += (LBReal)dpdy; lb->bz[x] += (LBReal)dpdz;
    }
  slb_mark_bodyforce(lb);
  slb_trace(lb, "zerobf");
}

/* reference src/lbobjs.c:623-643 */
void vset(LBSys lb, int i, int j, int k, LBReal vx, LBReal vy, LBReal vz) {
  long x;
  if (i >= 0 && i < lb->esi && j >= 0 && j < lb->esj && k >= 0 && k < lb->esk) {
    x = slb_node(lb, i, j, k);
    if (lb->obj[x] != NULL) {
      lb->ux[x] = lb->rho0 * vx / 12.0;
      lb->uy[x] = lb->rho0 * vy / 12.0;
      lb->uz[x] = lb->rho0 * vz / 12.0;
      slb_mark_wallvel(lb);
    }
  }
  slb_trace(lb, "vset");
}

/* reference src/lbobjs.c:648-655 */
int countfluid(LBSys lb) {
  long x;
  int count = 0;
  for (x = 0; x < lb->nnodes; x++) if (lb->obj[x] == NULL) count++;
  if (slb_verbosity & TRACE_ROUTINE_EXITS) printf("LB %i : countfluid done, = %i\n", lb->step, count);
  return count;
}

/* reference src/lbobjs.c:660-663 */
void syncobjs(LBSys lb) {
  makemask(lb);
  slb_state(lb)->nfluid = countfluid(lb);
  lb->changed_objects = 0;
  slb_mark_geometry(lb);
  slb_trace(lb, "syncobjs");
}

/* reference src/lbobjs.c:671-714 */
int countmask(LBSys lb, char *type) {
  long x;
  int q, count = 0, faces;
  switch (type[0]) {
    case 'a': case 'l': faces = 0; break;
    case 'f': case 's': faces = 1; break;
    default: printf("countmask: expected 'links' or 'faces'\n"); return 0;
  }
  for (x = 0; x < lb->nnodes; x++) {
    int m = lb->mask[x];
    if (m <= 0) continue;
    for (q = 1; q < (faces ? 7 : 15); q++)
      if (m & (1 << (q - 1))) count += faces ? 1 : lb->w[q];
  }
  slb_trace(lb, "countmask");
  return count;
}
