/*
 * ogs_oracle.c -- CPU oracle for the single-rank ogs gather-scatter path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA product
 * path is compared against, and the CPU baseline that bench.py times beside
 * it.  Nothing in dawgs_gb300/ links, loads or calls it; only tests/,
 * __graft_entry__.smoke() and bench.py (cpu_baseline leg and
 * `--impl reference`) do.
 *
 * It restates, in plain C with the same OpenMP row loops, the host
 * implementation of libParanumal's ogs library as vendored by paranumal/dawgs:
 *
 *   setup   libs/ogs/ogsSetup.cpp:69-190   ogsBase_t::Setup (zero ids skipped,
 *                                           Unsigned takes |id|)
 *           libs/ogs/ogsSetup.cpp:192-331  FindSharedNodes (grouping by |id|,
 *                                           `unique` flagging, gather_defined)
 *           libs/ogs/ogsSetup.cpp:333-433  ConstructSharedNodes (row numbering
 *                                           by first appearance in local order,
 *                                           positive groups first)
 *           libs/ogs/ogsSetup.cpp:569-683  LocalSignedSetup  (N and T maps)
 *           libs/ogs/ogsSetup.cpp:686-776  LocalUnsignedSetup (N aliases T)
 *   ops     libs/ogs/ogsOperator.cpp:36-55   Op_Add/Mul/Max/Min (identities
 *                                             0, 1, -max, +max)
 *           libs/ogs/ogsOperator.cpp:60-97   Gather
 *           libs/ogs/ogsOperator.cpp:206-238 Scatter
 *           libs/ogs/ogsOperator.cpp:311-360 GatherScatter
 *
 * One documented deviation: with `unique`, the reference keeps one member of
 * each id group positive, picked with rand() over an unstably sorted group
 * (ogsSetup.cpp:264-275).  Here the member with the lowest local index is
 * kept.  The choice changes which ids are flipped and the N maps of a Signed
 * unique handle, but not Sym GatherScatter, Gather(Trans) or Scatter(NoTrans),
 * which read the T maps only.
 *
 * Parity pin: the restatement is checked against gslib built from the
 * reference tree (3rdParty/gslib, the reference's own `-cc` checker), see
 * oracle/Makefile and tests/test_oracle_pin.py.
 *
 * Integer Add/Mul wrap modulo 2^bits (computed in unsigned arithmetic), which
 * is what the reference's `gv += v` on int does on every target it runs on.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { OR_FLOAT = 0, OR_DOUBLE = 1, OR_INT32 = 2, OR_INT64 = 3 };    /* ogs.hpp:179 */
enum { OR_ADD = 0, OR_MUL = 1, OR_MAX = 2, OR_MIN = 3 };             /* ogs.hpp:186 */
enum { OR_SYM = 0, OR_NOTRANS = 1, OR_TRANS = 2 };                   /* ogs.hpp:189 */
enum { OR_UNSIGNED = 0, OR_SIGNED = 1 };                             /* ogs.hpp:195 */

typedef struct {
  int64_t N;            /* local nodes (length of ids) */
  int kind, unique;
  int gather_defined;   /* every id group has exactly one positive member */
  int64_t NlocalP;      /* rows with a positive member = NrowsN */
  int64_t NlocalT;      /* all rows = NrowsT */
  int64_t Ngather, NgatherGlobal;
  int64_t nnzT, nnzN;
  int32_t *rowStartsT, *colIdsT;
  int32_t *rowStartsN, *colIdsN;  /* alias the T maps for Unsigned */
} oracle_ogs;

static int64_t iabs64(int64_t x) { return x < 0 ? -x : x; }

/* LSD radix sort of (key, payload) pairs by key, stable, 8 bits per pass. */
static void radix_sort_pairs(int64_t n, uint64_t *key, int64_t *val) {
  uint64_t *k2 = (uint64_t*)malloc((size_t)(n ? n : 1) * sizeof(uint64_t));
  int64_t *v2 = (int64_t*)malloc((size_t)(n ? n : 1) * sizeof(int64_t));
  uint64_t maxk = 0;
  for (int64_t i = 0; i < n; ++i) if (key[i] > maxk) maxk = key[i];
  for (int shift = 0; shift < 64 && (maxk >> shift) != 0; shift += 8) {
    int64_t cnt[257];
    memset(cnt, 0, sizeof(cnt));
    for (int64_t i = 0; i < n; ++i) cnt[((key[i] >> shift) & 255u) + 1]++;
    for (int b = 0; b < 256; ++b) cnt[b + 1] += cnt[b];
    for (int64_t i = 0; i < n; ++i) {
      int64_t p = cnt[(key[i] >> shift) & 255u]++;
      k2[p] = key[i];
      v2[p] = val[i];
    }
    memcpy(key, k2, (size_t)n * sizeof(uint64_t));
    memcpy(val, v2, (size_t)n * sizeof(int64_t));
  }
  free(k2);
  free(v2);
}

void oracle_free(oracle_ogs *h) {
  if (!h) return;
  if (h->rowStartsN != h->rowStartsT) free(h->rowStartsN);
  if (h->colIdsN != h->colIdsT) free(h->colIdsN);
  free(h->rowStartsT);
  free(h->colIdsT);
  memset(h, 0, sizeof(*h));
}

/* Returns 0 on success, 1 for an invalid option set (ogsSetup.cpp:98-100),
 * 2 for sizes beyond 32-bit device indices (types.h:59-63). */
int oracle_setup(oracle_ogs *h, int64_t N, int64_t *ids, int kind, int unique) {
  memset(h, 0, sizeof(*h));
  if (kind != OR_UNSIGNED && kind != OR_SIGNED) return 1;
  if (kind == OR_UNSIGNED && unique) return 1;
  if (N < 0 || N > INT32_MAX) return 2;
  h->N = N; h->kind = kind; h->unique = unique;

  /* ogsSetup.cpp:103-121 -- squeeze out zero ids */
  int64_t Nids = 0;
  for (int64_t n = 0; n < N; ++n) if (ids[n] != 0) Nids++;
  int64_t *loc = (int64_t*)malloc((size_t)(Nids ? Nids : 1) * sizeof(int64_t));
  int64_t *base = (int64_t*)malloc((size_t)(Nids ? Nids : 1) * sizeof(int64_t));
  Nids = 0;
  for (int64_t n = 0; n < N; ++n) {
    if (ids[n] != 0) {
      loc[Nids] = n;
      base[Nids] = (kind == OR_UNSIGNED) ? iabs64(ids[n]) : ids[n];
      Nids++;
    }
  }

  /* Group by |baseId|: a stable sort keeps members in ascending local order. */
  uint64_t *key = (uint64_t*)malloc((size_t)(Nids ? Nids : 1) * sizeof(uint64_t));
  int64_t *ord = (int64_t*)malloc((size_t)(Nids ? Nids : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < Nids; ++i) { key[i] = (uint64_t)iabs64(base[i]); ord[i] = i; }
  radix_sort_pairs(Nids, key, ord);

  /* FindSharedNodes (ogsSetup.cpp:252-301) and ConstructSharedNodes
   * (ogsSetup.cpp:352-385): per group, `unique` flagging, the positive-count
   * check behind gather_defined, and the group sign. */
  int64_t *grp = (int64_t*)malloc((size_t)(Nids ? Nids : 1) * sizeof(int64_t));
  unsigned char *gpos = (unsigned char*)malloc((size_t)(Nids ? Nids : 1));
  int64_t Ngroups = 0;
  int is_unique = 1;
  for (int64_t s = 0; s < Nids;) {
    int64_t e = s + 1;
    while (e < Nids && key[e] == key[s]) e++;
    if (unique) {
      const int64_t b = (int64_t)key[s];
      for (int64_t i = s; i < e; ++i) base[ord[i]] = -b;
      base[ord[s]] = b;  /* lowest local index stays positive */
    }
    int positive = 0;
    for (int64_t i = s; i < e; ++i) if (base[ord[i]] > 0) positive++;
    if (positive != 1) is_unique = 0;
    gpos[Ngroups] = positive > 0;
    for (int64_t i = s; i < e; ++i) grp[ord[i]] = Ngroups;
    Ngroups++;
    s = e;
  }
  h->gather_defined = is_unique;

  /* ogsSetup.cpp:409-433 -- rows numbered by first appearance in local order;
   * groups with a positive member take rows [0,NlocalP), the rest follow. */
  int64_t NlocalP = 0;
  for (int64_t g = 0; g < Ngroups; ++g) NlocalP += gpos[g];
  int64_t *rowOf = (int64_t*)malloc((size_t)(Ngroups ? Ngroups : 1) * sizeof(int64_t));
  for (int64_t g = 0; g < Ngroups; ++g) rowOf[g] = -1;
  int64_t cntP = 0, cntT = NlocalP;
  for (int64_t i = 0; i < Nids; ++i) {
    const int64_t g = grp[i];
    if (rowOf[g] == -1) rowOf[g] = gpos[g] ? cntP++ : cntT++;
  }
  h->NlocalP = NlocalP;
  h->NlocalT = Ngroups;
  h->Ngather = NlocalP;          /* NlocalP + NhaloP, NhaloP = 0 at one rank */
  h->NgatherGlobal = NlocalP;    /* Allreduce over one rank */

  /* ogsSetup.cpp:140-141 -- write flipped signs back when unique */
  if (unique) {
    for (int64_t i = 0; i < Nids; ++i) ids[loc[i]] = base[i];
  }

  /* LocalSignedSetup / LocalUnsignedSetup: counts, prefix sums, then colIds
   * filled in ascending local order (ogsSetup.cpp:590-663, 698-758). */
  const int64_t R = Ngroups;
  h->rowStartsT = (int32_t*)calloc((size_t)R + 1, sizeof(int32_t));
  for (int64_t i = 0; i < Nids; ++i) h->rowStartsT[rowOf[grp[i]] + 1]++;
  for (int64_t r = 0; r < R; ++r) h->rowStartsT[r + 1] += h->rowStartsT[r];
  h->nnzT = h->rowStartsT[R];
  h->colIdsT = (int32_t*)malloc((size_t)(h->nnzT ? h->nnzT : 1) * sizeof(int32_t));
  int32_t *fill = (int32_t*)calloc((size_t)R + 1, sizeof(int32_t));
  for (int64_t i = 0; i < Nids; ++i) {
    const int64_t r = rowOf[grp[i]];
    h->colIdsT[h->rowStartsT[r] + fill[r]++] = (int32_t)loc[i];
  }
  if (kind == OR_UNSIGNED) {
    h->rowStartsN = h->rowStartsT;
    h->colIdsN = h->colIdsT;
    h->nnzN = h->nnzT;
  } else {
    h->rowStartsN = (int32_t*)calloc((size_t)R + 1, sizeof(int32_t));
    for (int64_t i = 0; i < Nids; ++i)
      if (base[i] > 0) h->rowStartsN[rowOf[grp[i]] + 1]++;
    for (int64_t r = 0; r < R; ++r) h->rowStartsN[r + 1] += h->rowStartsN[r];
    h->nnzN = h->rowStartsN[R];
    h->colIdsN = (int32_t*)malloc((size_t)(h->nnzN ? h->nnzN : 1) * sizeof(int32_t));
    memset(fill, 0, ((size_t)R + 1) * sizeof(int32_t));
    for (int64_t i = 0; i < Nids; ++i) {
      if (base[i] > 0) {
        const int64_t r = rowOf[grp[i]];
        h->colIdsN[h->rowStartsN[r] + fill[r]++] = (int32_t)loc[i];
      }
    }
  }
  free(fill); free(rowOf); free(gpos); free(grp); free(ord); free(key);
  free(base); free(loc);
  return 0;
}

/* ---- operators (ogsOperator.cpp:36-55) ---------------------------------- */
#define OP_ADD_F(a, b) ((a) += (b))
#define OP_MUL_F(a, b) ((a) *= (b))
#define OP_ADD_I(UT, a, b) ((a) = (__typeof__(a))((UT)(a) + (UT)(b)))
#define OP_MUL_I(UT, a, b) ((a) = (__typeof__(a))((UT)(a) * (UT)(b)))
#define OP_MAX(a, b) ((a) = ((b) > (a)) ? (b) : (a))
#define OP_MIN(a, b) ((a) = ((b) < (a)) ? (b) : (a))

/* Expand BODY(T, INIT, OPSTMT) for one (type, op). */
#define OR_DISPATCH(type, op, BODY)                                               \
  switch (type) {                                                                 \
  case OR_FLOAT:                                                                  \
    switch (op) {                                                                 \
    case OR_ADD: BODY(float, 0.0f, OP_ADD_F) break;                              \
    case OR_MUL: BODY(float, 1.0f, OP_MUL_F) break;                              \
    case OR_MAX: BODY(float, -FLT_MAX, OP_MAX) break;                            \
    default:     BODY(float, FLT_MAX, OP_MIN) break;                             \
    } break;                                                                      \
  case OR_DOUBLE:                                                                 \
    switch (op) {                                                                 \
    case OR_ADD: BODY(double, 0.0, OP_ADD_F) break;                              \
    case OR_MUL: BODY(double, 1.0, OP_MUL_F) break;                              \
    case OR_MAX: BODY(double, -DBL_MAX, OP_MAX) break;                           \
    default:     BODY(double, DBL_MAX, OP_MIN) break;                            \
    } break;                                                                      \
  case OR_INT32:                                                                  \
    switch (op) {                                                                 \
    case OR_ADD: BODY(int32_t, 0, OP_ADD_I32) break;                             \
    case OR_MUL: BODY(int32_t, 1, OP_MUL_I32) break;                             \
    case OR_MAX: BODY(int32_t, -INT32_MAX, OP_MAX) break;                        \
    default:     BODY(int32_t, INT32_MAX, OP_MIN) break;                         \
    } break;                                                                      \
  default:                                                                        \
    switch (op) {                                                                 \
    case OR_ADD: BODY(int64_t, 0, OP_ADD_I64) break;                             \
    case OR_MUL: BODY(int64_t, 1, OP_MUL_I64) break;                             \
    case OR_MAX: BODY(int64_t, -INT64_MAX, OP_MAX) break;                        \
    default:     BODY(int64_t, INT64_MAX, OP_MIN) break;                         \
    } break;                                                                      \
  }
#define OP_ADD_I32(a, b) OP_ADD_I(uint32_t, a, b)
#define OP_MUL_I32(a, b) OP_MUL_I(uint32_t, a, b)
#define OP_ADD_I64(a, b) OP_ADD_I(uint64_t, a, b)
#define OP_MUL_I64(a, b) OP_MUL_I(uint64_t, a, b)

/* ogsOperator.cpp:60-97 -- NoTrans reads the N maps over NrowsN rows,
 * otherwise the T maps over NrowsT rows. */
void oracle_gather(const oracle_ogs *h, void *gv, const void *v, int K,
                   int type, int op, int trans) {
  const int64_t Nrows = (trans == OR_NOTRANS) ? h->NlocalP : h->NlocalT;
  const int32_t *rs = (trans == OR_NOTRANS) ? h->rowStartsN : h->rowStartsT;
  const int32_t *ci = (trans == OR_NOTRANS) ? h->colIdsN : h->colIdsT;
#define GATHER_BODY(T, INIT, OPF)                                    \
  {                                                                  \
    const T *vp = (const T*)v;                                       \
    T *gp = (T*)gv;                                                  \
    _Pragma("omp parallel for schedule(static)")                    \
    for (int64_t n = 0; n < Nrows; ++n) {                            \
      const int64_t s = rs[n], e = rs[n + 1];                        \
      for (int k = 0; k < K; ++k) {                                  \
        T val = INIT;                                                \
        for (int64_t g = s; g < e; ++g) OPF(val, vp[k + (int64_t)ci[g] * K]); \
        gp[k + n * K] = val;                                         \
      }                                                              \
    }                                                                \
  }
  OR_DISPATCH(type, op, GATHER_BODY)
#undef GATHER_BODY
}

/* ogsOperator.cpp:206-238 -- Trans writes through the N maps (NrowsN rows),
 * otherwise the T maps (NrowsT rows).  A plain element copy. */
void oracle_scatter(const oracle_ogs *h, void *v, const void *gv, int K,
                    int type, int trans) {
  const int64_t Nrows = (trans == OR_TRANS) ? h->NlocalP : h->NlocalT;
  const int32_t *rs = (trans == OR_TRANS) ? h->rowStartsN : h->rowStartsT;
  const int32_t *ci = (trans == OR_TRANS) ? h->colIdsN : h->colIdsT;
  const size_t sz = (type == OR_DOUBLE || type == OR_INT64) ? 8 : 4;
#define SCATTER_BODY(UT)                                                  \
  {                                                                       \
    UT *vp = (UT*)v;                                                      \
    const UT *gp = (const UT*)gv;                                         \
    _Pragma("omp parallel for schedule(static)")                         \
    for (int64_t n = 0; n < Nrows; ++n) {                                 \
      for (int64_t g = rs[n]; g < rs[n + 1]; ++g)                         \
        for (int k = 0; k < K; ++k) vp[k + (int64_t)ci[g] * K] = gp[k + n * K]; \
    }                                                                     \
  }
  if (sz == 8) SCATTER_BODY(uint64_t) else SCATTER_BODY(uint32_t)
#undef SCATTER_BODY
}

/* ogsOperator.cpp:311-360 -- Trans: gather T, scatter N, NrowsN rows;
 * Sym: T and T, NrowsT rows; NoTrans: gather N, scatter T, NrowsT rows. */
void oracle_gather_scatter(const oracle_ogs *h, void *v, int K, int type,
                           int op, int trans) {
  int64_t Nrows;
  const int32_t *grs, *gci, *srs, *sci;
  if (trans == OR_TRANS) {
    Nrows = h->NlocalP; grs = h->rowStartsT; gci = h->colIdsT; srs = h->rowStartsN; sci = h->colIdsN;
  } else if (trans == OR_SYM) {
    Nrows = h->NlocalT; grs = h->rowStartsT; gci = h->colIdsT; srs = h->rowStartsT; sci = h->colIdsT;
  } else {
    Nrows = h->NlocalT; grs = h->rowStartsN; gci = h->colIdsN; srs = h->rowStartsT; sci = h->colIdsT;
  }
#define GS_BODY(T, INIT, OPF)                                                 \
  {                                                                           \
    T *vp = (T*)v;                                                            \
    _Pragma("omp parallel for schedule(static)")                             \
    for (int64_t n = 0; n < Nrows; ++n) {                                     \
      for (int k = 0; k < K; ++k) {                                           \
        T val = INIT;                                                         \
        for (int64_t g = grs[n]; g < grs[n + 1]; ++g) OPF(val, vp[k + (int64_t)gci[g] * K]); \
        for (int64_t s = srs[n]; s < srs[n + 1]; ++s) vp[k + (int64_t)sci[s] * K] = val; \
      }                                                                       \
    }                                                                         \
  }
  OR_DISPATCH(type, op, GS_BODY)
#undef GS_BODY
}

/* Accessors for the ctypes wrapper. */
int64_t oracle_sizeof_handle(void) { return (int64_t)sizeof(oracle_ogs); }

void oracle_counts(const oracle_ogs *h, int64_t *out) {
  out[0] = h->N; out[1] = h->NlocalP; out[2] = h->NlocalT; out[3] = h->Ngather;
  out[4] = h->NgatherGlobal; out[5] = h->nnzT; out[6] = h->nnzN;
  out[7] = h->gather_defined;
}

void oracle_maps(const oracle_ogs *h, int32_t *rsT, int32_t *ciT, int32_t *rsN, int32_t *ciN) {
  memcpy(rsT, h->rowStartsT, ((size_t)h->NlocalT + 1) * sizeof(int32_t));
  memcpy(ciT, h->colIdsT, (size_t)h->nnzT * sizeof(int32_t));
  memcpy(rsN, h->rowStartsN, ((size_t)h->NlocalT + 1) * sizeof(int32_t));
  memcpy(ciN, h->colIdsN, (size_t)h->nnzN * sizeof(int32_t));
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
