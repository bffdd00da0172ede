/*
 * gsref_shim.c -- flat C entry points over gslib, built from the reference
 * tree's own 3rdParty/gslib sources (see oracle/Makefile) into
 * oracle/_ref/libgsref.so.
 *
 * TEST INFRASTRUCTURE ONLY: gslib is the reference's own correctness checker
 * for this path (dawgsGS.cpp:34-71 sets it up with gs_setup(..., gs_auto) and
 * dawgsMain.cpp:351-352 takes gs_vec(..., gs_double, gs_add, 0, ...) as the
 * golden result).  tests/ use it to pin the C restatement in ogs_oracle.c and
 * tests/golden/make_golden.py records its outputs as fixtures.  gslib is
 * compiled single-rank with MPI undefined (gslib src/comm.h:64-71).
 */
#include <stddef.h>
#include <stdlib.h>
#include <stdint.h>
#include "c99.h"
#include "name.h"
#include "fail.h"
#include "types.h"
#include "comm.h"
#include "mem.h"
#include "gs_defs.h"
#include "gs.h"

/* dtype codes follow ogs::Type: 0 float, 1 double, 2 int32, 3 int64 */
static gs_dom dom_of(int type) {
  switch (type) {
  case 0: return gs_float;
  case 1: return gs_double;
  case 2: return gs_int;
  default: return gs_long_long;
  }
}
/* op codes follow ogs::Op: 0 add, 1 mul, 2 max, 3 min */
static gs_op op_of(int op) {
  switch (op) {
  case 0: return gs_add;
  case 1: return gs_mul;
  case 2: return gs_max;
  default: return gs_min;
  }
}

void *gsref_setup(const int64_t *ids, int64_t n, int unique) {
  struct comm c;
  comm_init(&c, 0);
  slong *id = tmalloc(slong, n ? n : 1);
  for (int64_t i = 0; i < n; ++i) id[i] = (slong)ids[i];
  struct gs_data *g = gs_setup(id, (uint)n, &c, unique, gs_auto, 0);
  free(id);
  comm_free(&c);
  return g;
}

void gsref_gs(void *v, int type, int op, int transpose, void *g) {
  gs(v, dom_of(type), op_of(op), (unsigned)transpose, (struct gs_data*)g, 0);
}

void gsref_gs_vec(void *v, int k, int type, int op, int transpose, void *g) {
  gs_vec(v, (unsigned)k, dom_of(type), op_of(op), (unsigned)transpose, (struct gs_data*)g, 0);
}

void gsref_gs_many(void **vs, int k, int type, int op, int transpose, void *g) {
  gs_many((void *const*)vs, (unsigned)k, dom_of(type), op_of(op), (unsigned)transpose,
          (struct gs_data*)g, 0);
}

void gsref_unique(int64_t *ids, int64_t n) {
  struct comm c;
  comm_init(&c, 0);
  slong *id = tmalloc(slong, n ? n : 1);
  for (int64_t i = 0; i < n; ++i) id[i] = (slong)ids[i];
  gs_unique(id, (uint)n, &c);
  for (int64_t i = 0; i < n; ++i) ids[i] = (int64_t)id[i];
  free(id);
  comm_free(&c);
}

void gsref_free(void *g) { gs_free((struct gs_data*)g); }
