/*
 * ogs_c.h -- C ABI of the GB300 gather-scatter library (libdawgs_ogs.so).
 *
 * Drop-in for the single-rank hot path of libParanumal's ogs library as used
 * by paranumal/dawgs: ogs::ogs_t::Setup / GatherScatter / Gather / Scatter
 * (include/ogs.hpp:216-345 of the reference) over the CSR maps built by
 * ogsBase_t::Setup (libs/ogs/ogsSetup.cpp:69-190) and applied by
 * ogsOperator_t (libs/ogs/ogsOperator.cpp).  The reference exposes only C++
 * templates; every entry point below replaces one of those calls and keeps
 * its argument meaning.  Plain pointers and sizes only; device pointers are
 * CUDA device addresses, `stream` is a cudaStream_t (NULL = legacy default).
 *
 * Errors never cross the ABI as exceptions: each call returns an ogs_status
 * and ogs_last_error_string() gives the message of the calling thread's last
 * failure (the reference aborts with LIBP_ABORT, include/utils.hpp:57-76).
 *
 * Operations are asynchronous on `stream` unless the name ends in _host.  A
 * handle's maps are immutable after setup, so device-buffer calls on one
 * handle from several streams and threads are safe.  The _host calls share
 * the handle's device staging buffer: a lock in the handle serialises them
 * (each returns only after its stream has synchronised), and they allocate
 * that buffer on first use unless ogs_reserve_host made it at setup time.
 */
#ifndef OGS_C_H
#define OGS_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ogs_handle_s *ogs_handle;

typedef enum {
  OGS_OK = 0,
  OGS_EINVAL = 1,    /* bad argument or option set */
  OGS_ENOMEM = 2,    /* host or device allocation failed */
  OGS_EDEVICE = 3,   /* CUDA runtime error (message in ogs_last_error_string) */
  OGS_ETIMEOUT = 4,  /* a bounded wait ran out (ogs_server_wait_for) */
  OGS_ERANGE = 5,    /* sizes beyond 32-bit device indices or a stated limit */
  OGS_EUNDEFINED = 6 /* Gather/Scatter on a handle whose gather is not well-defined */
} ogs_status;

/* ogs::Type, include/ogs.hpp:179 of the reference */
typedef enum { OGS_FLOAT = 0, OGS_DOUBLE = 1, OGS_INT32 = 2, OGS_INT64 = 3 } ogs_type;
/* ogs::Op, include/ogs.hpp:186 */
typedef enum { OGS_ADD = 0, OGS_MUL = 1, OGS_MAX = 2, OGS_MIN = 3 } ogs_op;
/* ogs::Transpose, include/ogs.hpp:189 */
typedef enum { OGS_SYM = 0, OGS_NOTRANS = 1, OGS_TRANS = 2 } ogs_transpose;
/* ogs::Method, include/ogs.hpp:192 -- accepted and ignored at one rank */
typedef enum { OGS_AUTO = 0, OGS_PAIRWISE = 1, OGS_CRYSTALROUTER = 2, OGS_ALLTOALL = 3 } ogs_method;
/* ogs::Kind, include/ogs.hpp:195 (Halo is not part of the single-rank path) */
typedef enum { OGS_UNSIGNED = 0, OGS_SIGNED = 1, OGS_HALO = 2 } ogs_kind;

/* setup flags for ogs_setup_ex */
#define OGS_SETUP_VERBOSE   1u  /* print the reference's "ogs Setup Time" line */
#define OGS_SETUP_HOST_ONLY 2u  /* build host maps only; no device memory, no ops */
/* Where the N/T maps are built (the result is the same either way).  With
 * neither flag, a handle that is not host-only of at least
 * OGS_DEVICE_MAPS_MIN_N local nodes builds them on the GPU. */
#define OGS_SETUP_DEVICE_MAPS 4u /* sort and scan on the GPU; not with HOST_ONLY */
#define OGS_SETUP_HOST_MAPS   8u /* hash-table pass on the host */
#define OGS_DEVICE_MAPS_MIN_N 65536

typedef struct {
  int64_t N;              /* local nodes (ogsBase_t::N) */
  int64_t Ngather;        /* positive gathered rows, NlocalP + NhaloP (ogsBase.hpp:51) */
  int64_t NgatherGlobal;  /* = Ngather at one rank (ogsBase.hpp:56) */
  int64_t NlocalP;        /* rows with a positive member = NrowsN */
  int64_t NlocalT;        /* all rows = NrowsT */
  int64_t nnzT, nnzN;     /* entries of the T and N maps */
  int32_t gather_defined; /* 1 when every id group has exactly one positive member */
  int32_t kind, unique;
  int32_t max_degree;     /* largest row of the T map */
} ogs_counts;

typedef struct {
  int64_t rows_by_degree[9]; /* [d] rows of exact degree d (1..8); [0] rows above 8 */
  int64_t nnz_general;       /* entries in rows above degree 8 */
  int64_t ntiles;            /* 256-thread block tiles of the whole map (one-CTA-per-tile kernels) */
  int64_t device_bytes;      /* device memory held by the handle's maps */
  int64_t nphases;           /* slices of the host-buffer pipeline (at most 32) */
  int64_t phases[32][4];     /* per slice: lowest and highest node it touches, end of its
                                host->device chunk, end of the nodes final after it */
  int64_t nwarp_tiles;       /* warp tiles (32 lanes x 8 entries, exact degree): the work
                                items of the GatherScatter/Gather/Scatter launches */
  int64_t ngeneral_tiles;    /* tiles of rows above degree 8 */
  int64_t phase_rows[32][2]; /* per slice: end of the gathered rows final after it, end of the
                                gathered rows it and the earlier slices read */
} ogs_layout_stats;

/* ogs_t::Setup (include/ogs.hpp:221-228; libs/ogs/ogsSetup.cpp:69-190).
 * ids[N] are global ids (0 = does not participate).  With unique=1 (Signed
 * only) the ids are rewritten in place: one member of each group keeps a
 * positive id (the member with the lowest local index), the others are
 * negated (ogsSetup.cpp:138-141, 264-275).  Unsigned with unique=1 is
 * rejected (ogsSetup.cpp:98-100).  method is accepted and ignored. */
ogs_status ogs_setup(ogs_handle *out, int64_t N, int64_t *ids, int kind, int method,
                     int unique, int verbose);
ogs_status ogs_setup_ex(ogs_handle *out, int64_t N, int64_t *ids, int kind, int unique,
                        unsigned flags);
/* ogsBase_t::Free (libs/ogs/ogsSetup.cpp:849-859). NULL is accepted. */
ogs_status ogs_free(ogs_handle h);

/* ogs_t::GatherScatter(deviceMemory<T> o_v, k, op, trans)
 * (include/ogs.hpp:244-247; libs/ogs/ogs.cpp:39-123 ->
 * ogsOperator.cpp:311-360 semantics).  d_v holds k interleaved components
 * per node: component c of node n at d_v[c + n*k]. */
ogs_status ogs_gather_scatter(ogs_handle h, void *d_v, int k, int type, int op, int trans,
                              void *stream);
/* k separate arrays d_vs[0..k-1] of N values each (gslib's gs_many layout,
 * 3rdParty/gslib/src/gs.c:1354; ogs itself has no counterpart). */
ogs_status ogs_gather_scatter_many(ogs_handle h, void *const *d_vs, int k, int type, int op,
                                   int trans, void *stream);
/* ogs_t::Gather(deviceMemory<T> o_gv, o_v, k, op, trans) (include/ogs.hpp:285-289;
 * libs/ogs/ogs.cpp:202-298; ogsOperator.cpp:60-97).  d_gv has k*Ngather values
 * (Trans/Sym) -- rows NlocalP..NlocalT of an ill-defined handle are never
 * produced because Gather requires gather_defined (ogsSetup.cpp:861-864). */
ogs_status ogs_gather(ogs_handle h, void *d_gv, const void *d_v, int k, int type, int op,
                      int trans, void *stream);
/* ogs_t::Scatter(deviceMemory<T> o_v, o_gv, k, trans) (include/ogs.hpp:325-328;
 * libs/ogs/ogs.cpp:392-488; ogsOperator.cpp:206-238). */
ogs_status ogs_scatter(ogs_handle h, void *d_v, const void *d_gv, int k, int type, int trans,
                       void *stream);

/* Host-buffer overloads: ogs_t::GatherScatter/Gather/Scatter(memory<T> ...)
 * (include/ogs.hpp:232-236, 268-273, 309-313).  The work runs on the GPU:
 * the buffers are copied to a device staging area owned by the handle, the
 * kernel runs on `stream`, results are copied back, and the call returns
 * after `stream` has synchronised.  With page-locked buffers the copies and
 * the kernels run as a pipeline of up to 8 slices (copy in, compute and copy
 * out overlap); pageable buffers take one copy each way. */
ogs_status ogs_gather_scatter_host(ogs_handle h, void *v, int k, int type, int op, int trans,
                                   void *stream);
ogs_status ogs_gather_host(ogs_handle h, void *gv, const void *v, int k, int type, int op,
                           int trans, void *stream);
ogs_status ogs_scatter_host(ogs_handle h, void *v, const void *gv, int k, int type, int trans,
                            void *stream);

/* Reserve the device staging buffer and the copy streams and events of the
 * _host calls for fields of k components of `type`, so that no later _host
 * call on this handle with a field no larger (k*sizeof) allocates anything
 * (the reference allocates its exchange buffers in every call,
 * libs/ogs/ogs.cpp:53).  Covers GatherScatter, Gather and Scatter.  Calling
 * it again with a larger field grows the buffer; with a smaller one it does
 * nothing.  OGS_ENOMEM leaves the handle usable, without a buffer. */
ogs_status ogs_reserve_host(ogs_handle h, int k, int type);

/* ogs_gather_scatter_host without any device allocation.  No counterpart in
 * the reference: it exists for callers that must not have a library allocate
 * device memory once they are running -- latency-critical loops (cudaMalloc
 * and cudaFree synchronise the device), programs whose device memory belongs
 * to a framework's caching allocator, services with a fixed memory footprint.
 * The field is staged in a 32 MiB device array built into the library (held on
 * every device that loads it, until exit) instead of a cudaMalloc'd buffer;
 * fields larger than 32 MiB (N*k*sizeof(T)) are rejected with OGS_ERANGE.
 * The first call on each device looks the array's address up (set-up); make
 * that first call before any stream capture begins.  All calls share the one
 * array: calls that overlap on the GPU race.  Nothing in it needs to start
 * at zero: each call copies its whole field in before the kernel reads it.
 * The array's address is that of the device's primary context: after a
 * cudaDeviceReset, do not call this entry point again in the process.
 * Same refusals and the same results as ogs_gather_scatter_host, bit for bit;
 * the size is checked first, so an oversized field gets OGS_ERANGE whatever
 * the handle. */
ogs_status ogs_gather_scatter_host_noalloc(ogs_handle h, void *v, int k, int type, int op, int trans,
                                           void *stream);

/* Counts of ogsBase_t (include/ogs/ogsBase.hpp:50-58). */
ogs_status ogs_get_counts(ogs_handle h, ogs_counts *out);
/* Host copies of the CSR maps of ogsOperator_t (include/ogs/ogsOperator.hpp:47-57):
 * rowStartsT/N[NlocalT+1], colIdsT[nnzT], colIdsN[nnzN].  Any pointer may be NULL. */
ogs_status ogs_get_maps(ogs_handle h, int32_t *rowStartsT, int32_t *colIdsT,
                        int32_t *rowStartsN, int32_t *colIdsN);
/* Degree buckets and tiles the kernels run over (no reference counterpart). */
ogs_status ogs_get_layout_stats(ogs_handle h, ogs_layout_stats *out);
/* Column and row ids that the kernels found outside the handle's node and
 * row ranges since setup, counted by a library built with OGS_CHECK_BOUNDS=1
 * (a test build: each such id is replaced by 0 before any access); always 0
 * for a default build.  Synchronises with the device. */
ogs_status ogs_checked_id_errors(ogs_handle h, uint64_t *count);

/* ---- pieces of the multi-rank path that run on the device ----
 * An operator over caller-built CSR maps: the reference's ogsOperator_t
 * (include/ogs/ogsOperator.hpp:40-120), of which its multi-rank setup makes
 * gatherLocal, gatherHalo (libs/ogs/ogsSetup.cpp:569-776) and the exchange's
 * postmpi (libs/ogs/ogsAllToAll.cpp:255-331).  The T map (rowStartsT[NrowsT+1],
 * colIdsT) is required; colIds lie in [0, N).  rowStartsN == NULL makes the N
 * map the T map (Unsigned); otherwise rowStartsN has NrowsT+1 entries, rows at
 * and above NrowsN are empty and each row's N members are a subsequence of its
 * T members.  The handle takes ogs_gather / ogs_scatter / ogs_gather_scatter
 * (and the _host, _many forms) like one from ogs_setup, with no
 * gather-defined check (an operator has none); GatherScatter and Scatter are
 * refused when a local node sits in two rows.  ogs_gather may run in place
 * (d_gv == d_v) when no row reads an entry another row's result overwrites:
 * postmpi's maps (row n = own entry n, then received entries) are such.
 * flags: OGS_SETUP_HOST_ONLY or 0. */
ogs_status ogs_setup_maps(ogs_handle *out, int64_t N, int64_t NrowsN, int64_t NrowsT,
                          const int32_t *rowStartsN, const int32_t *colIdsN,
                          const int32_t *rowStartsT, const int32_t *colIdsT, unsigned flags);
/* Send-buffer packing, out[n*k+c] = q[ids[n]*k+c] for n < N: the reference's
 * extract kernel (libs/ogs/okl/ogsKernels.okl:167-177) as the all-to-all
 * exchange runs it before sending (libs/ogs/ogsAllToAll.cpp:126-131).
 * Device pointers; asynchronous on `stream`. */
ogs_status ogs_extract(int64_t N, int k, int type, const int32_t *d_ids, const void *d_q, void *d_out,
                       void *stream);

/* ---- halo_t: Exchange and Combine of the halo rows ----
 * libParanumal's halo_t (include/ogs.hpp:346-397; libs/ogs/ogsHalo.cpp:39-359).
 * Exchange gives every copy of a halo row its owner's value; Combine gives
 * the owner the sum over all copies.  The library runs the device steps on
 * the caller's stream -- the gatherHalo Gather into the halo buffer (or, for
 * a halo made from a gather, a copy of the gathered vector's halo rows) and
 * the Scatter back -- and calls the caller's exchange between them: the MPI
 * step that moves the halo buffer between ranks (ogsExchange_t::Start/Finish).
 * At one rank the halo has no rows and a NULL exchange is the reference's. */
typedef struct ogs_halo_s *ogs_halo;
/* The exchange object: start(user, d_buf, k, type, trans, stream) runs after
 * the halo buffer's rows [0, NhaloP) (Exchange, trans = OGS_NOTRANS) or
 * [0, NhaloT) (Combine, OGS_TRANS) are queued on `stream`; finish(...) must
 * leave rows [NhaloP, NhaloT) holding the owners' values (Exchange) or rows
 * [0, NhaloP) the sums (Combine) before the Scatter that follows on `stream`.
 * d_buf has room for k*(NhaloT + Nrecv) values.  Either may be NULL. */
typedef ogs_status (*ogs_exchange_fn)(void *user, void *d_buf, int k, int type, int trans, void *stream);
typedef struct {
  ogs_exchange_fn start, finish;
  void *user;
} ogs_exchange;
typedef struct {
  int64_t N;        /* entries of the vectors Exchange/Combine act on */
  int64_t NlocalT;  /* local rows before the halo rows (a halo from a gather) */
  int64_t NhaloP;   /* halo rows this rank owns */
  int64_t NhaloT;   /* all halo rows */
  int64_t Nhalo;    /* NhaloT - NhaloP: rows received from their owners (ogsSetup.cpp:63) */
  int64_t Nrecv;    /* extra rows of the halo buffer for the exchange's received entries */
  int32_t gathered; /* made from a gather (halo_t::SetupFromGather) */
  int32_t reserved;
} ogs_halo_counts;
/* halo_t::Setup (ogsSetup.cpp:55-64) at one rank: every nonzero id group must
 * have exactly one positive member (OGS_EINVAL otherwise, ogsSetup.cpp:286-288);
 * no group is shared with another rank, so the halo has no rows.  No device
 * memory is used. */
ogs_status ogs_halo_setup(ogs_halo *out, int64_t N, const int64_t *ids, int method, int verbose);
/* A halo over the gatherHalo maps that the reference's multi-rank setup
 * builds (ogsSetup.cpp:569-776: NhaloP rows with an N member first, NhaloT rows
 * in all; N maps may be NULL for Unsigned), as in ogs_setup_maps; Nrecv rows of
 * extra buffer for the exchange.  flags: OGS_SETUP_HOST_ONLY or 0. */
ogs_status ogs_halo_setup_maps(ogs_halo *out, int64_t N, int64_t NhaloP, int64_t NhaloT,
                               const int32_t *rowStartsN, const int32_t *colIdsN,
                               const int32_t *rowStartsT, const int32_t *colIdsT, int64_t Nrecv,
                               unsigned flags);
/* halo_t::SetupFromGather (ogsSetup.cpp:888-913): the vectors are gathered
 * ones, NlocalT local rows then NhaloT halo rows (the NhaloP owned ones first). */
ogs_status ogs_halo_setup_from_gather(ogs_halo *out, int64_t NlocalT, int64_t NhaloP, int64_t NhaloT,
                                      int64_t Nrecv);
ogs_status ogs_halo_free(ogs_halo h);
ogs_status ogs_halo_get_counts(ogs_halo h, ogs_halo_counts *out);
/* Reserve the halo buffer for k components of `type` (the calls below then
 * allocate nothing for fields no larger) and return it (NULL when the halo
 * has no rows).  The reference allocates it in every Start (ogsHalo.cpp:47). */
ogs_status ogs_halo_reserve(ogs_halo h, int k, int type, void **d_buf);
/* Exchange / Combine of a device vector (k interleaved components), with
 * their Start/Finish halves (ogsHalo.cpp:39-143, 185-303). */
ogs_status ogs_halo_exchange(ogs_halo h, void *d_v, int k, int type, const ogs_exchange *x, void *stream);
ogs_status ogs_halo_exchange_start(ogs_halo h, void *d_v, int k, int type, const ogs_exchange *x,
                                   void *stream);
ogs_status ogs_halo_exchange_finish(ogs_halo h, void *d_v, int k, int type, const ogs_exchange *x,
                                    void *stream);
ogs_status ogs_halo_combine(ogs_halo h, void *d_v, int k, int type, const ogs_exchange *x, void *stream);
ogs_status ogs_halo_combine_start(ogs_halo h, void *d_v, int k, int type, const ogs_exchange *x,
                                  void *stream);
ogs_status ogs_halo_combine_finish(ogs_halo h, void *d_v, int k, int type, const ogs_exchange *x,
                                   void *stream);
/* Host-vector forms (ogsHalo.cpp:150-183, 311-355): staged through the
 * device; return after `stream` has synchronised. */
ogs_status ogs_halo_exchange_host(ogs_halo h, void *v, int k, int type, const ogs_exchange *x, void *stream);
ogs_status ogs_halo_combine_host(ogs_halo h, void *v, int k, int type, const ogs_exchange *x, void *stream);

/* ---- gslib-compatible entry points ----
 * gslib (3rdParty/gslib of the reference) is the gather-scatter that dawgs
 * checks ogs against (dawgsGS.cpp:34-105).  These calls give its single-rank
 * results on the GPU, bit for bit: gs_setup(id, n, comm, unique=0, method,
 * verbose) (gs.c:1441), gs(u, dom, op, transpose) (gs.c:1266), gs_vec
 * (gs.c:1322) and gs_many (gs.c:1354).  Negative ids are flagged; transpose 0
 * folds unflagged members and sends the result to every member, transpose 1
 * folds all and writes the unflagged ones; see ogs_gslib.cpp for the rules.
 * dom uses ogs_type codes; ops add, mul, max, min (no bpr).  Free with
 * ogs_free.  A gslib handle is not accepted by the ogs_* operations. */
ogs_status ogs_gslib_setup(ogs_handle *out, const int64_t *ids, int64_t n, unsigned flags);
ogs_status ogs_gslib_gs(ogs_handle h, void *d_u, int dom, int op, int transpose, void *stream);
ogs_status ogs_gslib_gs_vec(ogs_handle h, void *d_u, int vn, int dom, int op, int transpose, void *stream);
ogs_status ogs_gslib_gs_many(ogs_handle h, void *const *d_us, int vn, int dom, int op, int transpose,
                             void *stream);

/* ---- Batched gather-scatter: many meshes in one persistent launch ----
 * No reference counterpart (dawgs calls ogs_t::GatherScatter once per mesh,
 * dawgsMain.cpp:211-219).  Each entry applies the reference GatherScatter
 * semantics (ogsOperator.cpp:311-360) with its own op, transpose and k to its
 * own interleaved device field; the results equal one ogs_gather_scatter per
 * entry bit for bit.  All entries share one value type and device.  Entries
 * must not share a field buffer.  A batch call is one persistent launch over
 * the entries below a size threshold plus, for the entries at or above it,
 * the single-mesh kernel on parallel branches beside it (the threshold 0
 * puts every entry in the persistent launch). */
typedef struct ogs_batch_s *ogs_batch;
typedef struct {
  ogs_handle h;   /* mesh */
  void *d_v;      /* device field: k interleaved components per node */
  int32_t k;
  int32_t op;     /* ogs_op */
  int32_t trans;  /* ogs_transpose */
  int32_t reserved;
} ogs_batch_entry;
/* The choices the tuner makes (the reference hard-codes its launch shape:
 * blockSize 256 and 512-member row blocks, include/ogs/ogsOperator.hpp:121-123). */
typedef struct {
  int32_t block;        /* threads per CTA of the persistent launch: 128 or 256 */
  int32_t ctas_per_sm;  /* its CTAs per SM (0 = as many as fit) */
  int64_t solo_items;   /* entries with at least this many work items (warp tiles x k)
                           run alone on the single-mesh kernel (0 = none) */
  int32_t solo_streams; /* parallel branches those launches are spread over (1..8) */
  int32_t sms;          /* (out) SMs of the device */
  int32_t from_cache;   /* (out) the tuner took this from its cache */
  int32_t occupancy;    /* register budget of the persistent launch: 2 or 3 256-thread
                           CTAs per SM (0 = 2) */
  double ms;            /* (out) the tuner's time for one batch call, ms */
  int32_t pipeline;     /* persistent launch: 0 values in registers (one item in flight
                           per warp), 1 values staged by cp.async in shared memory (two
                           items in flight; 256-thread blocks) */
  int32_t reserved;
} ogs_batch_config;
#define OGS_BATCH_GRAPH 1u  /* capture the launch in a CUDA graph on first use, replay after */
ogs_status ogs_batch_create(ogs_batch *out, int type, const ogs_batch_entry *entries, int n, unsigned flags);
/* Point the entries at new fields (one per entry); synchronises `stream`. */
ogs_status ogs_batch_set_fields(ogs_batch b, void *const *d_vs, void *stream);
/* All entries' gather-scatters, asynchronously on `stream`. */
ogs_status ogs_batch_gather_scatter(ogs_batch b, void *stream);
ogs_status ogs_batch_get_config(ogs_batch b, ogs_batch_config *cfg);
/* Use this configuration (its outputs are ignored); synchronises `stream`. */
ogs_status ogs_batch_set_config(ogs_batch b, const ogs_batch_config *cfg, void *stream);
/* The tuner: times candidate configurations (pipeline x block size x register
 * budget x CTAs per SM of the persistent launch, then size thresholds x branches for the single-mesh
 * launches, then CTAs per SM again) on scratch copies of the fields -- the
 * caller's fields are read once and never written -- and keeps the fastest.
 * The choice is cached for the process under a key of the value type, the SM
 * count, the k range and the histogram of log2(warp tiles) over the entries;
 * a batch with the same key takes the cached choice without timing.
 * OGS_TUNE_NO_CACHE times anyway (and refreshes the cache). */
#define OGS_TUNE_NO_CACHE 1u
ogs_status ogs_batch_tune_ex(ogs_batch b, void *stream, unsigned flags, ogs_batch_config *chosen);
/* ogs_batch_tune_ex with flags 0; *chosen_grid = the persistent launch's CTAs. */
ogs_status ogs_batch_tune(ogs_batch b, void *stream, int *chosen_grid);
/* The tuner's cache key for entries of records[i] warp tiles and ks[i] components. */
ogs_status ogs_batch_tune_key(int type, int sms, int n, const int64_t *records, const int32_t *ks,
                              uint64_t *key);
ogs_status ogs_batch_tune_cache_clear(void);
/* Work items (warp tile x component) of all entries. */
ogs_status ogs_batch_items(ogs_batch b, int64_t *items);
ogs_status ogs_batch_free(ogs_batch b);

/* ---- Served gather-scatter: resident meshes, continuous batching ----
 * No reference counterpart.  Requests name a resident mesh and carry a host
 * field (k interleaved components per node), gather-scattered in place with
 * the request's op and transpose.  A worker thread, which never blocks on the
 * GPU, admits pending requests in arrival order -- skipping, within a window,
 * those whose device buffer does not fit the budget yet, with a bound on how
 * often one may be passed over -- and runs everything admitted since its last
 * turn as one batched launch per value type.  Small and large fields travel
 * on separate copy and compute streams, so small requests do not queue
 * behind a large one's copies, and requests arriving while others run are
 * launched at once beside them.  Each result equals ogs_gather_scatter_host
 * of that request alone, bit for bit.  Submit from any thread; the host field
 * must stay valid and untouched until the request completes or is
 * cancelled. */
typedef struct ogs_server_s *ogs_server;
typedef struct {
  int64_t field_budget_bytes; /* device memory for request fields (the HBM budget) */
  int32_t max_inflight;       /* requests admitted and not yet retired */
  int32_t max_batch;          /* requests per batched launch */
} ogs_server_config;
typedef struct {
  int32_t mesh;   /* from ogs_server_add_mesh */
  int32_t type;   /* ogs_type */
  int32_t k;
  int32_t op;     /* ogs_op */
  int32_t trans;  /* ogs_transpose */
  int32_t reserved;
  void *host;     /* k*N values, in place */
} ogs_server_request;
ogs_status ogs_server_create(ogs_server *out, const ogs_server_config *cfg);
/* Make a set-up handle resident (the server does not own it). */
ogs_status ogs_server_add_mesh(ogs_server s, ogs_handle h, int *mesh_id);
/* arrival: time on ogs_server_clock() the request arrived, or 0 for now; a
 * time in the future schedules the request: it is not admitted before then
 * (latency still counts from `arrival`). */
ogs_status ogs_server_submit(ogs_server s, const ogs_server_request *r, double arrival, int64_t *id);
/* n requests at once, ids *first_id .. *first_id+n-1; arrivals may be NULL
 * (all now).  Either every request is queued or none (bad request, OGS_ERANGE). */
ogs_status ogs_server_submit_many(ogs_server s, const ogs_server_request *rs, const double *arrivals,
                                  int64_t n, int64_t *first_id);
double ogs_server_clock(void);
/* Until the request is done or cancelled (OGS_EDEVICE if the server failed). */
ogs_status ogs_server_wait(ogs_server s, int64_t id);
/* The same, giving up after timeout_s seconds with OGS_ETIMEOUT (the request
 * carries on; wait again or cancel it). */
ogs_status ogs_server_wait_for(ogs_server s, int64_t id, double timeout_s);
/* Withdraw a request that has not been admitted yet: *cancelled = 1 and it
 * never runs (its host field is not touched); *cancelled = 0 when it is
 * already running or done, and it completes normally. */
ogs_status ogs_server_cancel(ogs_server s, int64_t id, int *cancelled);
/* 0 pending, 1 admitted (on the GPU), 2 done, 3 cancelled. */
ogs_status ogs_server_state(ogs_server s, int64_t id, int *state);
/* Until every submitted request is done or cancelled. */
ogs_status ogs_server_drain(ogs_server s);
/* Arrival and completion times (ogs_server_clock seconds; -1 = not done) of
 * requests first..first+n-1. */
ogs_status ogs_server_latencies(ogs_server s, int64_t first, int64_t n, double *arrival, double *done);
/* The same with the time each request's launch was enqueued (-1 = not yet);
 * any pointer may be NULL. */
ogs_status ogs_server_times(ogs_server s, int64_t first, int64_t n, double *arrival, double *launched,
                            double *done);
ogs_status ogs_server_counters(ogs_server s, int64_t *launches, int64_t *batched_requests);
/* The worker thread's own timing, for finding where a latency tail comes
 * from: long gaps between its passes mean it slept or was descheduled, long
 * launches or retire passes mean CUDA calls blocked. */
typedef struct {
  int64_t passes;            /* passes of the worker loop */
  int64_t gaps_over_1ms;     /* passes that began more than 1 ms after the previous one */
  int64_t launches_over_1ms; /* lane launches (copies, tables, kernels) that took over 1 ms of host time */
  double max_gap_ms;
  double max_launch_ms;
  double max_retire_ms;      /* longest pass over the completion events */
} ogs_server_stats;
ogs_status ogs_server_get_stats(ogs_server s, ogs_server_stats *out);
/* Finishes outstanding requests, then releases the server. */
ogs_status ogs_server_free(ogs_server s);

/* ---- Testing hooks (no reference counterpart) ----
 * Every device and page-locked host allocation of the library is counted;
 * ogs_debug_fail_alloc(n) makes the n-th allocation from now fail as if the
 * memory were exhausted (n = 0 turns it off), so the OGS_ENOMEM paths can be
 * tested without exhausting a GPU.  ogs_debug_allocations reports the blocks
 * and bytes the library holds (any pointer may be NULL). */
ogs_status ogs_debug_fail_alloc(int64_t nth);
ogs_status ogs_debug_allocations(int64_t *device_blocks, int64_t *device_bytes, int64_t *host_blocks,
                                 int64_t *host_bytes);

/* Message of the calling thread's last failed call ("" if none). */
const char *ogs_last_error_string(void);
/* Library version, major*10000 + minor*100 + patch. */
int ogs_version(void);

#ifdef __cplusplus
}
#endif
#endif /* OGS_C_H */
