/* petsc_lite.c -- implementation of the single-rank PETSc/MPI stand-in described
 * in include/petsc_lite.h.  TEST INFRASTRUCTURE ONLY (oracle pinning). */
#include "petsc_lite.h"
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

struct _p_ISLocalToGlobalMapping {
  PetscInt *idx;
};

struct _p_DM {
  PetscInt NX, NY;
  PetscInt dof;          /* values per node: 1, or 3 for the Stokes solution DMDA (vx, vy, p) */
  int xperiodic;         /* DM_BOUNDARY_PERIODIC in x (nodalFields.c:11-19) */
  struct _p_ISLocalToGlobalMapping *ltog;  /* built on first request */
};

struct _p_Vec {
  DM dm;
  int is_local;          /* 1: (NX+4)*(NY+4) ghosted layout, 0: NX*NY */
  PetscInt n;
  PetscScalar *data;
  PetscScalar **rows;    /* row pointers handed out by DMDAVecGetArray */
};

static int g_quiet = 1;
void plite_set_quiet(int quiet) { g_quiet = quiet; }

PetscErrorCode plite_DMDACreate(PetscInt NX, PetscInt NY, DM *da) {
  *da = (DM)calloc(1, sizeof(struct _p_DM));
  if (!*da) return 1;
  (*da)->NX = NX;
  (*da)->NY = NY;
  (*da)->dof = 1;
  return 0;
}

void plite_DMDASetPeriodicX(DM da, int periodic) { da->xperiodic = periodic ? 1 : 0; }

PetscErrorCode plite_DMDACreateDOF(PetscInt NX, PetscInt NY, PetscInt dof, DM *da) {
  PetscErrorCode e = plite_DMDACreate(NX, NY, da);
  if (!e) (*da)->dof = dof;
  return e;
}

PetscErrorCode plite_DMDestroy(DM *da) {
  if (*da && (*da)->ltog) {
    free((*da)->ltog->idx);
    free((*da)->ltog);
  }
  free(*da);
  *da = NULL;
  return 0;
}

PetscErrorCode DMDAGetCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n,
                              PetscInt *p) {
  if (x) *x = 0;
  if (y) *y = 0;
  if (z) *z = 0;
  if (m) *m = da->NX;
  if (n) *n = da->NY;
  if (p) *p = 1;
  return 0;
}

static PetscErrorCode vec_new(DM da, int is_local, Vec *v) {
  Vec w = (Vec)calloc(1, sizeof(struct _p_Vec));
  if (!w) return 1;
  w->dm = da;
  w->is_local = is_local;
  w->n = (is_local ? (da->NX + 4) * (da->NY + 4) : da->NX * da->NY) * da->dof;
  w->data = (PetscScalar *)calloc((size_t)w->n, sizeof(PetscScalar));
  if (!w->data) { free(w); return 1; }
  *v = w;
  return 0;
}

PetscErrorCode DMCreateGlobalVector(DM da, Vec *v) { return vec_new(da, 0, v); }
PetscErrorCode DMCreateLocalVector(DM da, Vec *v) { return vec_new(da, 1, v); }
PetscErrorCode DMGetGlobalVector(DM da, Vec *v) { return vec_new(da, 0, v); }
PetscErrorCode DMGetLocalVector(DM da, Vec *v) { return vec_new(da, 1, v); }
PetscErrorCode DMRestoreGlobalVector(DM da, Vec *v) { (void)da; return VecDestroy(v); }
PetscErrorCode DMRestoreLocalVector(DM da, Vec *v) { (void)da; return VecDestroy(v); }

PetscErrorCode VecDuplicate(Vec a, Vec *b) { return vec_new(a->dm, a->is_local, b); }

PetscErrorCode VecDestroy(Vec *v) {
  if (!v || !*v) return 0;
  free((*v)->data);
  free((*v)->rows);
  free(*v);
  *v = NULL;
  return 0;
}

PetscErrorCode VecGetArray(Vec v, PetscScalar **a) { *a = v->data; return 0; }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a) { (void)v; *a = NULL; return 0; }
PetscErrorCode VecGetSize(Vec v, PetscInt *n) { *n = v->n; return 0; }

PetscErrorCode VecZeroEntries(Vec v) {
  memset(v->data, 0, (size_t)v->n * sizeof(PetscScalar));
  return 0;
}

PetscErrorCode VecSet(Vec v, PetscScalar a) {
  for (PetscInt i = 0; i < v->n; ++i) v->data[i] = a;
  return 0;
}

PetscErrorCode VecCopy(Vec x, Vec y) {
  if (x->n != y->n) return 60;
  memcpy(y->data, x->data, (size_t)x->n * sizeof(PetscScalar));
  return 0;
}

/* y = y + alpha*x */
PetscErrorCode VecAXPY(Vec y, PetscScalar alpha, Vec x) {
  if (x->n != y->n) return 60;
  for (PetscInt i = 0; i < y->n; ++i) y->data[i] = y->data[i] + alpha * x->data[i];
  return 0;
}

/* z = alpha*x + beta*y + gamma*z, with PETSc's alpha==1 shortcut: z = x + beta*y + gamma*z */
PetscErrorCode VecAXPBYPCZ(Vec z, PetscScalar alpha, PetscScalar beta, PetscScalar gamma, Vec x, Vec y) {
  if (x->n != z->n || y->n != z->n) return 60;
  PetscScalar *zz = z->data;
  const PetscScalar *xx = x->data, *yy = y->data;
  if (alpha == 1.0) {
    for (PetscInt i = 0; i < z->n; ++i) zz[i] = xx[i] + beta * yy[i] + gamma * zz[i];
  } else if (gamma == 1.0) {
    for (PetscInt i = 0; i < z->n; ++i) zz[i] = alpha * xx[i] + beta * yy[i] + zz[i];
  } else if (gamma == 0.0) {
    for (PetscInt i = 0; i < z->n; ++i) zz[i] = alpha * xx[i] + beta * yy[i];
  } else {
    for (PetscInt i = 0; i < z->n; ++i) zz[i] = alpha * xx[i] + beta * yy[i] + gamma * zz[i];
  }
  return 0;
}

/* w = x ./ y, zero where y == 0 */
PetscErrorCode VecPointwiseDivide(Vec w, Vec x, Vec y) {
  if (x->n != w->n || y->n != w->n) return 60;
  for (PetscInt i = 0; i < w->n; ++i) {
    PetscScalar d = y->data[i];
    w->data[i] = (d != 0.0) ? x->data[i] / d : 0.0;
  }
  return 0;
}

PetscErrorCode VecSum(Vec v, PetscScalar *s) {
  PetscScalar acc = 0.0;
  for (PetscInt i = 0; i < v->n; ++i) acc += v->data[i];
  *s = acc;
  return 0;
}

PetscErrorCode VecView(Vec v, PetscViewer vw) { (void)v; (void)vw; return 0; }

PetscErrorCode DMGlobalToLocalBegin(DM da, Vec g, InsertMode mode, Vec l) {
  (void)mode;
  if (g->is_local || !l->is_local) return 62;
  const PetscInt NX = da->NX, NY = da->NY, W = NX + 4;
  for (PetscInt j = 0; j < NY; ++j) {
    PetscScalar *row = l->data + (size_t)(j + 2) * W + 2;
    const PetscScalar *src = g->data + (size_t)j * NX;
    memcpy(row, src, (size_t)NX * sizeof(PetscScalar));
    if (da->xperiodic) {  /* ghost columns -2, -1, NX, NX+1 hold their periodic images */
      row[-2] = src[NX - 2];
      row[-1] = src[NX - 1];
      row[NX] = src[0];
      row[NX + 1] = src[1];
    }
  }
  return 0;
}
PetscErrorCode DMGlobalToLocalEnd(DM da, Vec g, InsertMode mode, Vec l) { (void)da; (void)g; (void)mode; (void)l; return 0; }

PetscErrorCode DMLocalToGlobalBegin(DM da, Vec l, InsertMode mode, Vec g) {
  if (g->is_local || !l->is_local) return 62;
  const PetscInt NX = da->NX, NY = da->NY, W = NX + 4;
  for (PetscInt j = 0; j < NY; ++j) {
    const PetscScalar *src = l->data + (size_t)(j + 2) * W + 2;
    PetscScalar *dst = g->data + (size_t)j * NX;
    if (mode == ADD_VALUES) {
      for (PetscInt i = 0; i < NX; ++i) dst[i] = dst[i] + src[i];
      if (da->xperiodic) {  /* ghost columns add into their periodic owners, after the interior */
        dst[NX - 2] = dst[NX - 2] + src[-2];
        dst[NX - 1] = dst[NX - 1] + src[-1];
        dst[0] = dst[0] + src[NX];
        dst[1] = dst[1] + src[NX + 1];
      }
    } else {
      memcpy(dst, src, (size_t)NX * sizeof(PetscScalar));
    }
  }
  return 0;
}
PetscErrorCode DMLocalToGlobalEnd(DM da, Vec l, InsertMode mode, Vec g) { (void)da; (void)l; (void)mode; (void)g; return 0; }

PetscErrorCode DMDAVecGetArray(DM da, Vec v, void *array) {
  const PetscInt NX = da->NX, NY = da->NY;
  const int g = v->is_local ? 2 : 0;
  const PetscInt W = NX + 2 * g, H = NY + 2 * g;
  if (!v->rows) {
    v->rows = (PetscScalar **)malloc((size_t)H * sizeof(PetscScalar *));
    if (!v->rows) return 1;
  }
  for (PetscInt r = 0; r < H; ++r) v->rows[r] = v->data + (size_t)r * W + g;
  *(PetscScalar ***)array = v->rows + g;
  return 0;
}
PetscErrorCode DMDAVecRestoreArray(DM da, Vec v, void *array) { (void)da; (void)v; *(PetscScalar ***)array = NULL; return 0; }
/* [j][i][dof] view of a global vector of a multi-dof DMDA (dof interleaved per node) */
PetscErrorCode DMDAVecGetArrayDOF(DM da, Vec v, void *array) {
  if (v->is_local) return 63;
  const PetscInt NX = da->NX, NY = da->NY, dof = da->dof;
  PetscScalar ***a = (PetscScalar ***)malloc((size_t)NY * sizeof(PetscScalar **));
  PetscScalar **cells = (PetscScalar **)malloc((size_t)NY * NX * sizeof(PetscScalar *));
  if (!a || !cells) return 1;
  for (PetscInt j = 0; j < NY; ++j) {
    a[j] = cells + (size_t)j * NX;
    for (PetscInt i = 0; i < NX; ++i) a[j][i] = v->data + ((size_t)j * NX + i) * dof;
  }
  *(PetscScalar ****)array = a;
  return 0;
}
PetscErrorCode DMDAVecRestoreArrayDOF(DM da, Vec v, void *array) {
  (void)da;
  (void)v;
  PetscScalar ***a = *(PetscScalar ****)array;
  if (a) {
    free(a[0]);
    free(a);
  }
  *(PetscScalar ****)array = NULL;
  return 0;
}

/* elementwise operations, as PETSc documents them (no fused multiply-add: the stand-in is
 * compiled with -ffp-contract=off) */
PetscErrorCode VecScale(Vec x, PetscScalar a) {
  for (PetscInt k = 0; k < x->n; ++k) x->data[k] = a * x->data[k];
  return 0;
}
PetscErrorCode VecShift(Vec x, PetscScalar a) {
  for (PetscInt k = 0; k < x->n; ++k) x->data[k] = x->data[k] + a;
  return 0;
}
PetscErrorCode VecPointwiseMult(Vec w, Vec x, Vec y) {
  for (PetscInt k = 0; k < w->n; ++k) w->data[k] = x->data[k] * y->data[k];
  return 0;
}
PetscErrorCode VecAYPX(Vec y, PetscScalar beta, Vec x) {  /* y = x + beta y */
  for (PetscInt k = 0; k < y->n; ++k) y->data[k] = x->data[k] + beta * y->data[k];
  return 0;
}
/* largest / smallest entry; NaN entries never win (comparisons with NaN are false) */
PetscErrorCode VecMax(Vec x, PetscInt *idx, PetscReal *v) {
  PetscReal m = -INFINITY;
  PetscInt at = -1;
  for (PetscInt k = 0; k < x->n; ++k)
    if (x->data[k] > m) {
      m = x->data[k];
      at = k;
    }
  if (idx) *idx = at;
  *v = m;
  return 0;
}
PetscErrorCode VecMin(Vec x, PetscInt *idx, PetscReal *v) {
  PetscReal m = INFINITY;
  PetscInt at = -1;
  for (PetscInt k = 0; k < x->n; ++k)
    if (x->data[k] < m) {
      m = x->data[k];
      at = k;
    }
  if (idx) *idx = at;
  *v = m;
  return 0;
}
/* scale component `field` of a dof-interleaved vector */
PetscErrorCode VecStrideScale(Vec v, PetscInt field, PetscScalar a) {
  const PetscInt dof = v->dm->dof;
  for (PetscInt k = field; k < v->n; k += dof) v->data[k] = v->data[k] * a;
  return 0;
}

/* ---- logging stages: exclusive wall time attributed to the top of the stack ---- */
#define PLITE_MAX_STAGES 64
#define PLITE_STACK 64
static int g_nstages = 0;
static double g_stage_sec[PLITE_MAX_STAGES];
static int g_stack[PLITE_STACK];
static int g_depth = 0;
static double g_last = 0.0;

static double now_sec(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

PetscErrorCode PetscLogStageRegister(const char *name, PetscLogStage *s) {
  (void)name;
  if (g_nstages >= PLITE_MAX_STAGES) return 1;
  *s = g_nstages++;
  return 0;
}

static void charge_top(void) {
  double t = now_sec();
  if (g_depth > 0) g_stage_sec[g_stack[g_depth - 1]] += t - g_last;
  g_last = t;
}

PetscErrorCode PetscLogStagePush(PetscLogStage s) {
  charge_top();
  if (g_depth < PLITE_STACK) g_stack[g_depth++] = s;
  return 0;
}

PetscErrorCode PetscLogStagePop(void) {
  charge_top();
  if (g_depth > 0) g_depth--;
  return 0;
}

double plite_stage_seconds(int stage) {
  return (stage >= 0 && stage < PLITE_MAX_STAGES) ? g_stage_sec[stage] : 0.0;
}

void plite_stage_reset(void) {
  memset(g_stage_sec, 0, sizeof(g_stage_sec));
  g_depth = 0;
  g_last = now_sec();
}

PetscErrorCode PetscPrintf(MPI_Comm c, const char *fmt, ...) {
  (void)c;
  if (g_quiet) return 0;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  return 0;
}
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm c, const char *fmt, ...) {
  (void)c;
  if (g_quiet) return 0;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  return 0;
}
PetscErrorCode PetscSynchronizedFlush(MPI_Comm c, ...) { (void)c; return 0; }

/* ---- random numbers ----
 * PETSCRAND48 objects draw from the C library's global drand48 stream, which PetscRandomSeed
 * seeds with srand48(seed) -- the documented behaviour of PETSc's rand48 type; the reference's
 * own drand48() calls (markers.c:651) share that stream.  Every other type gets a private
 * erand48 stream whose 48-bit state PetscRandomSetSeed sets to (seed << 16) | 0x330E.  Values
 * are lo + (hi - lo) * u with u uniform on [0, 1). */
struct _p_PetscRandom {
  double lo, hi;
  unsigned short state[3];
  unsigned long seed;
  int rand48;
};

PetscErrorCode PetscRandomCreate(MPI_Comm c, PetscRandom *r) {
  (void)c;
  *r = (PetscRandom)calloc(1, sizeof(struct _p_PetscRandom));
  if (!*r) return 1;
  (*r)->lo = 0.0;
  (*r)->hi = 1.0;
  return 0;
}
PetscErrorCode PetscRandomSetType(PetscRandom r, PetscRandomType t) {
  r->rand48 = t && strcmp(t, PETSCRAND48) == 0;
  return 0;
}
PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed) {
  r->seed = seed;
  r->state[0] = 0x330E;
  r->state[1] = (unsigned short)(seed & 0xFFFF);
  r->state[2] = (unsigned short)((seed >> 16) & 0xFFFF);
  return 0;
}
PetscErrorCode PetscRandomSeed(PetscRandom r) {
  if (r->rand48) srand48((long)r->seed);
  return 0;
}
PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscScalar lo, PetscScalar hi) {
  r->lo = lo;
  r->hi = hi;
  return 0;
}
PetscErrorCode PetscRandomGetValue(PetscRandom r, PetscScalar *v) {
  const double u = r->rand48 ? drand48() : erand48(r->state);
  *v = r->lo + (r->hi - r->lo) * u;
  return 0;
}
PetscErrorCode PetscRandomDestroy(PetscRandom *r) {
  free(*r);
  *r = NULL;
  return 0;
}

int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }

static size_t mpi_type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    default: return 1;
  }
}

int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
  (void)op;
  (void)c;
  if (s != r) memmove(r, s, (size_t)count * mpi_type_size(t));
  return 0;
}

int MPI_Sendrecv(const void *sb, int sc, MPI_Datatype st, int dest, int stag, void *rb, int rc, MPI_Datatype rt,
                 int src, int rtag, MPI_Comm c, MPI_Status *status) {
  (void)dest; (void)stag; (void)src; (void)rtag; (void)c; (void)status;
  size_t n = (size_t)sc * mpi_type_size(st);
  size_t m = (size_t)rc * mpi_type_size(rt);
  if (n > m) n = m;
  if (n) memmove(rb, sb, n);
  return 0;
}

/* ---- one-rank collectives and point-to-point ---- */
int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm c) {
  (void)rc; (void)rt; (void)c;
  memcpy(r, s, (size_t)sc * mpi_type_size(st));
  return 0;
}
int MPI_Gather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, int root, MPI_Comm c) {
  (void)rc; (void)rt; (void)root; (void)c;
  memcpy(r, s, (size_t)sc * mpi_type_size(st));
  return 0;
}
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c;
  return 1;  /* no other rank */
}
int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st) {
  (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st;
  return 1;
}

/* ---- viewers, bags, names, options: inert ---- */
PetscErrorCode PetscViewerASCIIOpen(MPI_Comm c, const char *n, PetscViewer *v) { (void)c; (void)n; *v = NULL; return 0; }
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm c, const char *n, PetscFileMode m, PetscViewer *v) {
  (void)c; (void)n; (void)m; *v = NULL; return 0;
}
PetscErrorCode PetscViewerMatlabOpen(MPI_Comm c, const char *n, PetscFileMode m, PetscViewer *v) {
  (void)c; (void)n; (void)m; *v = NULL; return 0;
}
PetscErrorCode PetscViewerCreate(MPI_Comm c, PetscViewer *v) { (void)c; *v = NULL; return 0; }
PetscErrorCode PetscViewerSetType(PetscViewer v, PetscViewerType t) { (void)v; (void)t; return 0; }
PetscErrorCode PetscViewerFileSetMode(PetscViewer v, PetscFileMode m) { (void)v; (void)m; return 0; }
PetscErrorCode PetscViewerFileSetName(PetscViewer v, const char *n) { (void)v; (void)n; return 0; }
PetscErrorCode PetscViewerSetFormat(PetscViewer v, PetscViewerFormat f) { (void)v; (void)f; return 0; }
PetscErrorCode PetscViewerMatlabPutArray(PetscViewer v, int m, int n, const PetscScalar *a, const char *nm) {
  (void)v; (void)m; (void)n; (void)a; (void)nm; return 0;
}
PetscErrorCode PetscViewerDestroy(PetscViewer *v) { if (v) *v = NULL; return 0; }
PetscErrorCode PetscObjectSetName(PetscObject o, const char *n) { (void)o; (void)n; return 0; }
PetscErrorCode DMView(DM d, PetscViewer v) { (void)d; (void)v; return 0; }
PetscErrorCode DMGetCoordinates(DM d, Vec *c) { (void)d; *c = NULL; return 1; }  /* no coordinates kept */
PetscErrorCode PetscOptionsGetBool(const char *pre, const char *name, PetscBool *v, PetscBool *set) {
  (void)pre; (void)name; (void)v;
  if (set) *set = PETSC_FALSE;
  return 0;
}

#include "petscbag.h"
struct _p_PetscBag { void *data; };
PetscErrorCode PetscBagCreate(MPI_Comm c, size_t sz, PetscBag *b) {
  (void)c;
  *b = (PetscBag)calloc(1, sizeof(struct _p_PetscBag));
  if (!*b) return 1;
  (*b)->data = calloc(1, sz ? sz : 1);
  return (*b)->data ? 0 : 1;
}
PetscErrorCode PetscBagGetData(PetscBag b, void **d) { *d = b->data; return 0; }
PetscErrorCode PetscBagRegisterScalar(PetscBag b, void *a, PetscScalar v, const char *n, const char *h) {
  (void)b; (void)n; (void)h;
  *(PetscScalar *)a = v;
  return 0;
}
PetscErrorCode PetscBagView(PetscBag b, PetscViewer v) { (void)b; (void)v; return 0; }
PetscErrorCode PetscBagDestroy(PetscBag *b) {
  if (*b) { free((*b)->data); free(*b); *b = NULL; }
  return 0;
}

/* ---- Mat ------------------------------------------------------------------------------ */
typedef struct {
  PetscInt n, cap;
  PetscInt *col;
  PetscScalar *val;
} MatRow;

struct _p_Mat {
  PetscInt nrows;
  MatRow *rows;
};

PetscErrorCode plite_MatCreate(PetscInt nrows, Mat *A) {
  Mat m = (Mat)calloc(1, sizeof(struct _p_Mat));
  if (!m) return 1;
  m->nrows = nrows;
  m->rows = (MatRow *)calloc((size_t)(nrows > 0 ? nrows : 1), sizeof(MatRow));
  if (!m->rows) { free(m); return 1; }
  *A = m;
  return 0;
}

PetscErrorCode MatDestroy(Mat *A) {
  if (!A || !*A) return 0;
  for (PetscInt r = 0; r < (*A)->nrows; ++r) {
    free((*A)->rows[r].col);
    free((*A)->rows[r].val);
  }
  free((*A)->rows);
  free(*A);
  *A = NULL;
  return 0;
}

/* PETSc keeps the nonzero pattern and zeroes the values */
PetscErrorCode MatZeroEntries(Mat A) {
  for (PetscInt r = 0; r < A->nrows; ++r)
    for (PetscInt k = 0; k < A->rows[r].n; ++k) A->rows[r].val[k] = 0.0;
  return 0;
}

static PetscErrorCode mat_set(Mat A, PetscInt r, PetscInt c, PetscScalar v, InsertMode mode) {
  if (r < 0 || c < 0) return 0;
  if (r >= A->nrows || c >= A->nrows) return 63;  /* PETSC_ERR_ARG_OUTOFRANGE */
  MatRow *row = &A->rows[r];
  for (PetscInt k = 0; k < row->n; ++k)
    if (row->col[k] == c) {
      row->val[k] = mode == ADD_VALUES ? row->val[k] + v : v;
      return 0;
    }
  if (row->n == row->cap) {
    PetscInt nc = row->cap ? 2 * row->cap : 8;
    PetscInt *ci = (PetscInt *)realloc(row->col, (size_t)nc * sizeof(PetscInt));
    if (!ci) return 55;
    row->col = ci;
    PetscScalar *vv = (PetscScalar *)realloc(row->val, (size_t)nc * sizeof(PetscScalar));
    if (!vv) return 55;
    row->val = vv;
    row->cap = nc;
  }
  row->col[row->n] = c;
  row->val[row->n] = v;  /* a new entry: INSERT and ADD both give v */
  row->n++;
  return 0;
}

PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt *rows, PetscInt n, const PetscInt *cols,
                            const PetscScalar *v, InsertMode mode) {
  for (PetscInt i = 0; i < m; ++i)
    for (PetscInt j = 0; j < n; ++j) {
      PetscErrorCode e = mat_set(A, rows[i], cols[j], v[i * n + j], mode);
      if (e) return e;
    }
  return 0;
}

PetscErrorCode MatSetValue(Mat A, PetscInt row, PetscInt col, PetscScalar v, InsertMode mode) {
  return mat_set(A, row, col, v, mode);
}

PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }

PetscErrorCode MatCopy(Mat A, Mat B, MatStructure s) {
  (void)s;
  if (A->nrows != B->nrows) return 60;
  for (PetscInt r = 0; r < A->nrows; ++r)
    for (PetscInt k = 0; k < A->rows[r].n; ++k) {
      PetscErrorCode e = mat_set(B, r, A->rows[r].col[k], A->rows[r].val[k], INSERT_VALUES);
      if (e) return e;
    }
  return 0;
}

PetscInt plite_MatGetCSR(Mat A, PetscInt **rowptr, PetscInt **cols, PetscScalar **vals) {
  PetscInt nnz = 0;
  for (PetscInt r = 0; r < A->nrows; ++r) nnz += A->rows[r].n;
  *rowptr = (PetscInt *)malloc((size_t)(A->nrows + 1) * sizeof(PetscInt));
  *cols = (PetscInt *)malloc((size_t)(nnz ? nnz : 1) * sizeof(PetscInt));
  *vals = (PetscScalar *)malloc((size_t)(nnz ? nnz : 1) * sizeof(PetscScalar));
  PetscInt at = 0;
  for (PetscInt r = 0; r < A->nrows; ++r) {
    (*rowptr)[r] = at;
    const MatRow *row = &A->rows[r];
    for (PetscInt k = 0; k < row->n; ++k) {  /* insertion sort by column */
      PetscInt c = row->col[k];
      PetscScalar v = row->val[k];
      PetscInt q = at;
      while (q > (*rowptr)[r] && (*cols)[q - 1] > c) {
        (*cols)[q] = (*cols)[q - 1];
        (*vals)[q] = (*vals)[q - 1];
        --q;
      }
      (*cols)[q] = c;
      (*vals)[q] = v;
      ++at;
    }
  }
  (*rowptr)[A->nrows] = at;
  return nnz;
}

PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt *idx, const PetscScalar *y, InsertMode mode) {
  for (PetscInt k = 0; k < n; ++k) {
    PetscInt i = idx[k];
    if (i < 0) continue;
    if (i >= v->n) return 63;
    v->data[i] = mode == ADD_VALUES ? v->data[i] + y[k] : y[k];
  }
  return 0;
}

PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar y, InsertMode mode) { return VecSetValues(v, 1, &i, &y, mode); }
PetscErrorCode VecAssemblyBegin(Vec v) { (void)v; return 0; }
PetscErrorCode VecAssemblyEnd(Vec v) { (void)v; return 0; }

PetscErrorCode DMGetLocalToGlobalMapping(DM da, ISLocalToGlobalMapping *map) {
  if (!da->ltog) {
    const PetscInt mg = da->NX + 4, ng = da->NY + 4;
    ISLocalToGlobalMapping m = (ISLocalToGlobalMapping)calloc(1, sizeof(*m));
    if (!m) return 55;
    m->idx = (PetscInt *)malloc((size_t)mg * ng * sizeof(PetscInt));
    if (!m->idx) { free(m); return 55; }
    for (PetscInt jl = 0; jl < ng; ++jl)
      for (PetscInt il = 0; il < mg; ++il) {
        const PetscInt i = il - 2, j = jl - 2;
        m->idx[il + mg * jl] = (i >= 0 && i < da->NX && j >= 0 && j < da->NY) ? j * da->NX + i : -1;
      }
    da->ltog = m;
  }
  *map = da->ltog;
  return 0;
}

PetscErrorCode ISLocalToGlobalMappingGetIndices(ISLocalToGlobalMapping map, const PetscInt **idx) {
  *idx = map->idx;
  return 0;
}

PetscErrorCode ISLocalToGlobalMappingRestoreIndices(ISLocalToGlobalMapping map, const PetscInt **idx) {
  (void)map;
  *idx = NULL;
  return 0;
}

PetscErrorCode DMDAGetGhostCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n,
                                   PetscInt *p) {
  if (x) *x = -2;
  if (y) *y = -2;
  if (z) *z = 0;
  if (m) *m = da->NX + 4;
  if (n) *n = da->NY + 4;
  if (p) *p = 1;
  return 0;
}
