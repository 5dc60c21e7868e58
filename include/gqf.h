/*
 * gqf.h -- C ABI of the GB300 quotient-filter engine (libgqf.so).
 *
 * Plain C: device pointers, sizes and an opaque CUDA stream (`void*`, NULL =
 * the legacy default stream, which is what the reference uses).  Every entry
 * point returns a gqf_status.  When `ms` is non-NULL the call is synchronous
 * like the reference API (it waits for the work, reports device-side errors
 * and stores the elapsed device time in *ms); when `ms` is NULL the work is
 * only enqueued on `stream` and device-side errors are collected later by
 * gqf_stream_status().
 *
 * Each declaration names the reference function it replaces
 * (owensgroup/GPUQuotientFilters, file:line).  The struct layouts are the
 * reference's own, so a filter made by either API can be used by the other.
 */
#ifndef GQF_H
#define GQF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gqf_status {
    GQF_OK = 0,
    GQF_ERR_ARG = 1,       /* bad q/r, null or unaligned pointer, negative count */
    GQF_ERR_FULL = 2,      /* layout needs more than (1<<q)*1.1 slots       */
    GQF_ERR_CUDA = 3,      /* a CUDA runtime call failed                    */
    GQF_ERR_TIMEOUT = 4,   /* a bounded device-side wait ran out            */
    GQF_ERR_NOMEM = 5,     /* workspace allocation failed                   */
    GQF_ERR_MISMATCH = 6,  /* mergeTwoFilters on filters of different q/r   */
    GQF_ERR_LIMIT = 7,     /* request larger than the fixed no-allocation scratch */
    GQF_ERR_FORMAT = 8,    /* serialized image: bad header, size or checksum */
    GQF_ERR_IO = 9         /* file could not be opened, read or written */
} gqf_status;

/* Standard quotient filter handle: identical to `struct quotient_filter`
 * (standardQuotientFilter/GPU_version/quotientFilter.cuh:25-31). */
typedef struct gqf_sqf {
    unsigned int qbits;
    unsigned int rbits;
    unsigned int bytesPerElement;
    unsigned char *table; /* device, calcNumSlotsGPU(q, r) bytes, 16-byte aligned
                           * (cudaMalloc gives 256); others return GQF_ERR_ARG */
} gqf_sqf;

/* Rank-and-select filter handle: identical to `struct
 * countingQuotientFilterGPU` (rankSelectQuotientFilter/GPU_version/
 * RSQF.cuh:32-37).  Blocks use the reference's packed layout
 * (RSQF.cuh:24-30): u8 offset, u64 occupieds, u64 runEnds,
 * u64 remainders[5] = 57 bytes, and gqf allocates one extra zeroed guard
 * block after the numBlocks logical ones. */
typedef struct gqf_rsqf {
    unsigned int qbits;
    unsigned int numBlocks;
    void *blocks;
} gqf_rsqf;

#define GQF_NOT_FOUND 0xFFFFFFFFu
#define GQF_RSQF_RBITS 5
#define GQF_RSQF_BLOCK_BYTES 57

/* ---------------- sizing and hashing (host only, no GPU needed) --------- */
/* calcNumSlotsGPU, quotientFilter.cu:37-42: table bytes for (q, r) */
size_t gqf_sqf_table_bytes(unsigned int q, unsigned int r);
/* (1<<q)*1.1 slots, the bound used by findRunStartGPU (quotientFilter.cu:174) */
unsigned int gqf_sqf_num_slots(unsigned int q);
/* Normal_APHash, quotientFilter.cu:134-149 */
unsigned int gqf_aphash(unsigned int value, unsigned int table_size);
/* calcNumBlocksGPU, RSQF.cu:27-30 */
size_t gqf_rsqf_num_blocks(unsigned int q);
/* MT19937 draws after init_genrand(seed) (mt19937ar.cpp:57,102), skipping
 * `skip` draws first: the reference drivers' key generator. */
void gqf_mt19937_fill(uint32_t seed, uint64_t skip, uint32_t *out, uint64_t n);
const char *gqf_status_string(int status);
/* Number of kernels this library has launched in this process
 * (instrumentation; no counterpart in the reference). */
unsigned long long gqf_kernel_launches(void);
/* latched device error for `stream` since the last call (waits for it) */
int gqf_stream_status(void *stream);
/* Scratch workspaces (no reference counterpart): every stream has its own,
 * grown on demand and kept, so calls on different streams may overlap on
 * the device.  reserve pre-grows a stream's workspace (a later call that
 * fits allocates nothing); release frees it after the stream drains. */
int gqf_workspace_reserve(void *stream, size_t bytes, size_t *reserved);
int gqf_workspace_release(void *stream);
/* Workspace bytes one gqf_sqf_insert / gqf_sqf_delete of n keys on a
 * filter of (q, r) needs. */
size_t gqf_sqf_update_workspace_bytes(unsigned int q, unsigned int r, int n);

/* ---------------- standard quotient filter ------------------------------ */
/* initFilterGPU, quotientFilter.cu:44-55.  Allocates and ZEROES the table
 * (the reference leaves it uninitialised; its callers memset it). */
int gqf_sqf_init(gqf_sqf *qf, unsigned int q, unsigned int r);
int gqf_sqf_free(gqf_sqf *qf);

/* bulkBuildSegmentedLayouts, quotientFilter.cu:1446-1559.  Rebuilds the
 * whole table from the n keys (clears it first). */
int gqf_sqf_bulk_build(const gqf_sqf *qf, int n, const uint32_t *d_keys,
                       int no_duplicates, void *stream, float *ms);

/* launchUnsortedLookups, quotientFilter.cu:359-381: d_out[i] = slot of
 * key i's remainder, or GQF_NOT_FOUND.  On one-byte slots a batch of at least
 * one query per 16 slots first transposes the table into a bit-plane mirror
 * (stream workspace, 32 bytes per 31 slots) and answers each query from two
 * of its 32-byte records. */
int gqf_sqf_lookup_unsorted(const gqf_sqf *qf, int n, const uint32_t *d_keys,
                            uint32_t *d_out, void *stream, float *ms);

/* launchSortedLookups, quotientFilter.cu:272-318: same results as the
 * unsorted lookup (input order).  Batches of at least one query per 16 slots
 * take the unsorted path above; smaller ones group the queries by table
 * region. */
int gqf_sqf_lookup_sorted(const gqf_sqf *qf, int n, const uint32_t *d_keys,
                          uint32_t *d_out, void *stream, float *ms);

/* insert, quotientFilter.cu:533-634: adds each key's fingerprint unless it
 * is already present. */
int gqf_sqf_insert(const gqf_sqf *qf, int n, const uint32_t *d_keys,
                   void *stream, float *ms);

/* superclusterDeletes, quotientFilter.cu:1202-1297: removes one stored copy
 * of each key's fingerprint. */
int gqf_sqf_delete(const gqf_sqf *qf, int n, const uint32_t *d_keys,
                   void *stream, float *ms);

/* insertViaMerge, quotientFilter.cu:1602-1742 (d_old/n_old are unused by
 * the algorithm, as in the reference :1604). */
int gqf_sqf_insert_via_merge(const gqf_sqf *qf, const uint32_t *d_old, int n_old,
                             const uint32_t *d_new, int n_new, int no_duplicates,
                             void *stream, float *ms);

/* mergeTwoFilters, quotientFilter.cu:1744-1891: qf1 := qf1 + qf2. */
int gqf_sqf_merge(const gqf_sqf *qf1, const gqf_sqf *qf2, int no_duplicates,
                  void *stream, float *ms);

/* Bulk build that allocates no device memory (no counterpart in the
 * reference).  It is for callers that cannot call cudaMalloc while they run:
 * a process whose own pool allocator reserved the GPU's memory at start-up,
 * a latency-critical stream where cudaMalloc/cudaFree's implicit device
 * synchronisation would stall other streams, or a service with a fixed
 * memory budget that must not grow after start-up.  The caller still owns
 * the filter table and the keys.  Scratch is a fixed array in the library's
 * device image (GQF_NOALLOC_SCRATCH_BYTES per GPU that loads the library,
 * held until the process exits); requests beyond GQF_NOALLOC_MAX_KEYS keys
 * or GQF_NOALLOC_MAX_Q quotient bits return GQF_ERR_LIMIT.  The first call
 * on a device looks up the array's device address, so make that first call
 * before any stream capture.  Every call on a device shares that device's
 * one array.  The library serialises calls from different host threads on
 * one device, and each call waits for its own work before it returns, so
 * calls only overlap on the GPU when one returned an error after enqueuing
 * work; calls whose work overlaps on the GPU race and corrupt each other's
 * results.  Device-side errors are returned like the timed entry points'. */
#define GQF_NOALLOC_MAX_KEYS (1u << 20)
#define GQF_NOALLOC_MAX_Q 22
#define GQF_NOALLOC_SCRATCH_BYTES (12u << 20)
int gqf_sqf_bulk_build_noalloc(const gqf_sqf *qf, int n, const uint32_t *d_keys,
                               int no_duplicates, void *stream);

/* Test support, no counterpart in the reference.  Runs the bulk build's
 * decoupled look-back (one warp per bucket) over nb host-given 64-bit bucket
 * descriptors -- [63:62] flag (0 unpublished, 1 aggregate, 2 inclusive),
 * aggregate: [61:31] items n, [30:0] end slot F from slot 0; inclusive:
 * [30:0] first slot after the bucket -- and stores each bucket's entry slot
 * in cin[b].  A wait on an unpublished descriptor is polled at most
 * spin_limit times; if any wait runs out the call returns GQF_ERR_TIMEOUT
 * (those buckets get cin 0) and the device stays usable.  Allocates, and
 * synchronises the device. */
int gqf_debug_lookback_probe(const unsigned long long *status, unsigned int nb, unsigned int spin_limit,
                             unsigned int *cin);

/* ---------------- rank-and-select quotient filter ----------------------- */
/* initCQFGPU, RSQF.cu:32-40 (zeroed blocks + one guard block) */
int gqf_rsqf_init(gqf_rsqf *cqf, unsigned int q);
int gqf_rsqf_free(gqf_rsqf *cqf);
/* insertGPU, RSQF.cu:882-988: d_ret[i] = slot of the i-th smallest
 * fingerprint of the batch, or -1 */
int gqf_rsqf_insert(const gqf_rsqf *cqf, int n, const uint32_t *d_keys,
                    int32_t *d_ret, void *stream, float *ms);
/* launchLookups, RSQF.cu:411-456 (slot or -1, in input order).  Batches of
 * at least one query per 16 slots are probed directly, smaller ones grouped
 * by block first. */
int gqf_rsqf_lookup_sorted(const gqf_rsqf *cqf, int n, const uint32_t *d_keys,
                           int32_t *d_out, void *stream, float *ms);
/* launchUnsortedLookups, RSQF.cu:540-563 */
int gqf_rsqf_lookup_unsorted(const gqf_rsqf *cqf, int n, const uint32_t *d_keys,
                             int32_t *d_out, void *stream, float *ms);

/* ---------------- rank-and-select filter with 8-bit remainders ---------- */
/* The same calls for the reference RSQF compiled with RBITS 8 (the
 * remainder width of RSQF.cuh:21 / RSQF.h:23, a compile-time constant
 * there): blocks of 81 bytes (u8 offset, u64 occupieds, u64 runEnds, u64
 * remainders[8]) plus the guard block.  Fingerprints have q + 8 bits, so
 * q <= 23; a gqf_rsqf handle made by gqf_rsqf8_init is used only with the
 * gqf_rsqf8_* calls. */
#define GQF_RSQF8_RBITS 8
#define GQF_RSQF8_BLOCK_BYTES 81
size_t gqf_rsqf8_num_blocks(unsigned int q);
int gqf_rsqf8_init(gqf_rsqf *cqf, unsigned int q);
int gqf_rsqf8_free(gqf_rsqf *cqf);
int gqf_rsqf8_insert(const gqf_rsqf *cqf, int n, const uint32_t *d_keys,
                     int32_t *d_ret, void *stream, float *ms);
int gqf_rsqf8_lookup_sorted(const gqf_rsqf *cqf, int n, const uint32_t *d_keys,
                            int32_t *d_out, void *stream, float *ms);
int gqf_rsqf8_lookup_unsorted(const gqf_rsqf *cqf, int n, const uint32_t *d_keys,
                              int32_t *d_out, void *stream, float *ms);

/* ---------------- batched filters (no counterpart in the reference) ----- */
/* Many independent standard filters built and queried together: one launch
 * of each pipeline kernel covers every filter of the batch (work lists of
 * scatter chunks, buckets and query chunks across all filters), and the
 * launch sequence is captured once into a CUDA graph.  A job bulk builds
 * its filter from n_build keys (as gqf_sqf_bulk_build; n_build == 0 leaves
 * the table as it is), then answers n_lookup unsorted lookups (as
 * gqf_sqf_lookup_unsorted).  All filters of a batch share r.  The batch
 * keeps the job pointers: run it again after refilling the same buffers.
 * Every filter that is rebuilt needs q >= the tuning's bucket bits. */
typedef struct gqf_sqf_job {
    gqf_sqf filter;
    int n_build;
    const uint32_t *d_build_keys;
    int n_lookup;
    const uint32_t *d_lookup_keys;
    uint32_t *d_results;
} gqf_sqf_job;
/* Launch shape of a batch (0 = default): bucket_bits = log2 quotients per
 * layout CTA (10..13, default 12); scatter_chunk = keys per scatter CTA
 * (2048, 8192 or 32768, default 8192).  The persistent pipeline's shape:
 * cta_threads (128 or 256, default 256) and items_per_thread (keys per
 * thread of a scatter chunk: 8 or 32, default 32); its layout threads own
 * 2^bucket_bits / cta_threads quotients each, 16 or 32 (other shapes leave
 * the persistent mode unavailable: GQF_ERR_ARG from gqf_batch_run). */
typedef struct gqf_batch_tuning {
    int bucket_bits;
    int scatter_chunk;
    int cta_threads;
    int items_per_thread;
} gqf_batch_tuning;
typedef struct gqf_batch gqf_batch;
int gqf_batch_create(gqf_batch **out, const gqf_sqf_job *jobs, int count, int no_duplicates,
                     const gqf_batch_tuning *tuning);
/* use_graph: GQF_BATCH_DIRECT (0) launches the pipeline's kernels on
 * `stream`; GQF_BATCH_GRAPH (1) replays them as one captured CUDA graph;
 * GQF_BATCH_PERSISTENT (2) runs the whole pipeline as ONE cooperative
 * kernel launch whose CTAs take work units from the same lists and meet at
 * grid barriers between the phases (bounded waits: GQF_ERR_TIMEOUT). */
#define GQF_BATCH_DIRECT 0
#define GQF_BATCH_GRAPH 1
#define GQF_BATCH_PERSISTENT 2
int gqf_batch_run(gqf_batch *batch, int use_graph, void *stream, float *ms);
int gqf_batch_tuning_of(const gqf_batch *batch, gqf_batch_tuning *out);
int gqf_batch_destroy(gqf_batch *batch);

/* ---------------- served filters (no counterpart in the reference) ------ */
/* A request loop over resident filters with continuous batching: requests
 * (a lookup, insert or delete batch on one filter, host key buffers) are
 * queued per filter; whenever a device stream slot frees up, the filter
 * whose oldest request waited longest gets an op made of all its queued
 * requests of that request's kind (consecutive same-kind requests coalesce;
 * the result is the one of applying them one by one).  Ops of different
 * filters run concurrently on separate streams, one op per filter at a
 * time, so every filter sees its requests in submission order.  The HBM
 * budget bounds tables + per-stream workspaces + staging: it fixes how many
 * streams (ops in flight) the server runs.  Key and result buffers must
 * stay valid until the request completes (pinned memory lets copies
 * overlap). */
enum { GQF_SERVE_LOOKUP = 0, GQF_SERVE_INSERT = 1, GQF_SERVE_DELETE = 2 };
typedef struct gqf_server_config {
    size_t hbm_budget_bytes; /* 0: no limit beyond the device's memory     */
    int max_streams;         /* concurrent ops at most (0: 8)              */
    int max_op_keys;         /* keys per coalesced op (0: 2^22)            */
    int coalesce;            /* 0: one request per op                      */
} gqf_server_config;
typedef struct gqf_completion {
    uint64_t id;
    int status;
    double submit_us, start_us, done_us; /* since the server started      */
} gqf_completion;
typedef struct gqf_server gqf_server;
int gqf_server_create(gqf_server **out, const gqf_sqf *filters, int nfilters, const gqf_server_config *cfg);
int gqf_server_submit(gqf_server *srv, int filter, int op, const uint32_t *keys, int n, uint32_t *results,
                      uint64_t *id);
/* completed requests since the last poll (at most max) */
int gqf_server_poll(gqf_server *srv, gqf_completion *out, int max, int *count);
/* waits until every submitted request has completed */
int gqf_server_drain(gqf_server *srv);
int gqf_server_info(const gqf_server *srv, int *streams, size_t *hbm_bytes);
int gqf_server_destroy(gqf_server *srv);

/* ---------------- serialization (no counterpart in the reference) ------- */
/* Checkpoint / restore of a filter as one host image: a 64-byte header
 * (magic "GQFSQF01" or "GQFRSQF1", format version, q, r, payload bytes,
 * FNV-1a-64 checksum of the payload; little-endian) followed by the raw
 * device table: the SQF slot array exactly as calcNumSlotsGPU sizes it, or
 * the RSQF's numBlocks packed 57-byte blocks (the guard block is not
 * stored).  Images restore bit-identically into a filter of the same q/r. */
#define GQF_IMAGE_HEADER_BYTES 64
size_t gqf_sqf_image_bytes(const gqf_sqf *qf);
size_t gqf_rsqf_image_bytes(const gqf_rsqf *cqf);
/* copy the filter into host memory `buf` of `cap` bytes (waits for `stream`) */
int gqf_sqf_save(const gqf_sqf *qf, void *buf, size_t cap, void *stream);
int gqf_rsqf_save(const gqf_rsqf *cqf, void *buf, size_t cap, void *stream);
/* allocate a filter (as gqf_sqf_init / gqf_rsqf_init) holding the image */
int gqf_sqf_load(gqf_sqf *qf, const void *buf, size_t len);
int gqf_rsqf_load(gqf_rsqf *cqf, const void *buf, size_t len);
int gqf_sqf_save_file(const gqf_sqf *qf, const char *path);
int gqf_rsqf_save_file(const gqf_rsqf *cqf, const char *path);
int gqf_sqf_load_file(gqf_sqf *qf, const char *path);
int gqf_rsqf_load_file(gqf_rsqf *cqf, const char *path);

#ifdef __cplusplus
}
#endif
#endif /* GQF_H */
