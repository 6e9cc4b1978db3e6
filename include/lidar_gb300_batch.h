/*
 * lidar_gb300_batch.h — prepared batches: scans uploaded once into HBM and re-executed, for
 * throughput measurement, CUDA-graph replay and the serving loop. These entry points have no
 * counterpart in the reference library (it processes one scan per call on the CPU); they run the
 * same launch sequence as lp_process_batch (lidar_gb300.h).
 */
#ifndef LIDAR_GB300_BATCH_H
#define LIDAR_GB300_BATCH_H

#include "lidar_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lp_batch lp_batch;

/* Plans the layout, allocates device memory and uploads the scans (host buffers must stay
 * valid for lp_batch_upload). A batch of 16 or more scans is split into up to eight parts (one per
 * 8 scans, dealt round-robin) that execute concurrently on their own streams, forked from and
 * joined into the context stream; results and their order are those of the unsplit batch. */
lp_status lp_batch_create(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans,
                          uint32_t nscans, lp_batch** out);
void lp_batch_destroy(lp_context* ctx, lp_batch* batch);
/* Copies the scans' host buffers to the device again (asynchronous on the context stream). */
lp_status lp_batch_upload(lp_context* ctx, lp_batch* batch);
/* Runs the whole pipeline on the device-resident inputs (asynchronous: complete when the context
 * stream reaches this point). */
lp_status lp_batch_execute(lp_context* ctx, lp_batch* batch);
/* Captures the launch sequence into a CUDA graph; later lp_batch_execute calls replay it. */
lp_status lp_batch_capture_graph(lp_context* ctx, lp_batch* batch);
/* Waits for the stream and copies every scan's results into outs[0..nscans). */
lp_status lp_batch_download(lp_context* ctx, lp_batch* batch, lp_scan_output* outs);
lp_status lp_context_synchronize(lp_context* ctx);
uint32_t lp_batch_points(const lp_batch* batch);
uint64_t lp_batch_device_bytes(const lp_batch* batch);
/* Mean device time of one execution over `iters` runs (CUDA events on the context stream);
 * flush_l2 writes a 512 MiB buffer before each run, outside the timed interval. */
lp_status lp_batch_time(lp_context* ctx, lp_batch* batch, uint32_t iters, int32_t flush_l2, float* ms_per_iter);
/* Per-kernel device times of one execution: names (name_len bytes each) and milliseconds for up
 * to cap launches in launch order; *count receives the number of launches. */
lp_status lp_batch_profile(lp_context* ctx, lp_batch* batch, char* names, uint32_t name_len, float* ms,
                           uint32_t cap, uint32_t* count);
/* Page-locked host memory (cudaMallocHost) for scan inputs and result buffers: the library's
 * copies to and from it run asynchronously at the host link's full rate, where pageable memory is
 * staged through a bounce buffer. Not zeroed. No counterpart in the reference (its callers own
 * plain std::vector buffers, which remain accepted everywhere). */
lp_status lp_host_alloc(uint64_t bytes, void** out);
void lp_host_free(void* p);

/* The kd-tree the outlier filter builds on the device for the cloud xyz (n points, stride floats
 * apart): per node position, x, y, z and the subtree size (as uint32 bits), n x 4 floats into
 * nodes_out. It equals the reference's KDTree::rebuild (kdtree.hpp:161-214) node for node; used by
 * the parity tests. No counterpart in the reference. */
lp_status lp_debug_kdtree(lp_context* ctx, const float* xyz, uint32_t stride, uint32_t n,
                          const lp_noise_remover_config* cfg, float* nodes_out);
/* Bounded waits giving up: kind 0 runs the device-wide prefix scan on a tile whose predecessor
 * never publishes (its ticket counter starts past tile 0), kind 1 waits on an mbarrier that never
 * completes; each polls `limit` times, then records the failure as the library's kernels do.
 * Returns LP_ERR_TIMEOUT with *gave_up != 0 when the wait gave up (the expected outcome), leaving
 * the context usable. For the failure-path tests; no counterpart in the reference. */
lp_status lp_debug_wait_timeout(lp_context* ctx, int32_t kind, uint32_t limit, uint32_t* gave_up);
/* Device evaluation of the library's correctly rounded binary32 functions (kind 0 atan2(a, b),
 * 1 atan(a), 2 exp(a), 3 the reference's atan2 approximation; 4, 5, 6 the same three functions
 * without their float-float first stage); used by the parity tests. */
lp_status lp_debug_math(lp_context* ctx, int32_t kind, const float* a, const float* b, uint32_t n, float* out);
/* Check of the float-float first stage of those functions against the binary64 / double-double
 * stages over `count` arguments starting at index `first` (kind 1 atan, 2 exp: the float with bits
 * first + i; kind 0 atan2: hashed pairs). stats[0] = decided by the first stage, stats[1] = left
 * to the later stages, stats[2] = decided differently (must be 0); *first_bad = lowest index of
 * such a difference (UINT64_MAX when none). */
lp_status lp_debug_math_sweep(lp_context* ctx, int32_t kind, uint64_t first, uint64_t count, uint64_t stats[3],
                              uint64_t* first_bad);

/* ------------------------------------------------------------------------------------------ */
/* Tuning: batch split and launch shapes chosen at run time, per batch bucket.                 */
/* No counterpart in the reference (it runs one scan at a time on one CPU thread).             */
/* ------------------------------------------------------------------------------------------ */
typedef struct lp_tuning
{
    uint32_t parts;            /* concurrent parts of a batch of 16 or more scans (1-8; 0: one per 8
                                  scans, at most 8); never more than the batch has scans */
    uint32_t balance_parts;    /* 0: scans dealt round-robin; 1: largest scan first to the part holding
                                  the fewest points */
    uint32_t hull_cta_min;     /* clusters of more members take a whole CTA of the hull kernel, smaller
                                  ones one warp (64-512) */
    uint32_t hull_ctas_per_sm; /* persistent hull CTAs per SM (1-4) */
    uint32_t cell_ctas_per_sm; /* polar-cell sort CTAs per SM (1-16) */
    uint32_t jcp_ctas_per_sm;  /* vote-weight CTAs per SM (1-16) */
} lp_tuning;

/* A batch's bucket: scan-count class (0: 1 scan, 1: 2-15, 2: 16-31, 3: 32-63, 4: 64 or more), and
 * the ring-count class (0: up to 32 rings, 1: up to 64, 2: more) and azimuth class (0: up to 1024
 * bins, 1: up to 2048, 2: more) that hold the most points of the batch. */
typedef struct lp_tuning_key
{
    uint32_t scans_class;
    uint32_t ring_class;
    uint32_t azimuth_class;
} lp_tuning_key;

typedef struct lp_tuning_table lp_tuning_table;

/* The compiled-in defaults (set by sweeps of the 64-scan mixed batch). */
void lp_tuning_default(lp_tuning* t);
/* LP_ERR_BAD_ARG unless every field lies in its range. */
lp_status lp_tuning_validate(const lp_tuning* t);
lp_status lp_tuning_key_of(const lp_scan_input* scans, uint32_t nscans, lp_tuning_key* out);
/* Host-side table bucket -> tuning (and the step time it was measured at). */
lp_status lp_tuning_table_create(lp_tuning_table** out);
void lp_tuning_table_destroy(lp_tuning_table* table);
lp_status lp_tuning_table_set(lp_tuning_table* table, const lp_tuning_key* key, const lp_tuning* tuning, float ms);
/* 1 and the entry when the bucket is in the table; 0 and the defaults when it is not. */
int32_t lp_tuning_table_get(const lp_tuning_table* table, const lp_tuning_key* key, lp_tuning* out, float* ms);
uint32_t lp_tuning_table_size(const lp_tuning_table* table);
/* Plain text, one bucket per line; load adds to (and overrides entries of) the table. */
lp_status lp_tuning_table_save(const lp_tuning_table* table, const char* path);
lp_status lp_tuning_table_load(lp_tuning_table* table, const char* path);
/* The context keeps a copy: batches created afterwards (lp_batch_create, lp_process_batch, the
 * serving loop) take their bucket's entry, the defaults where there is none. */
lp_status lp_context_set_tuning_table(lp_context* ctx, const lp_tuning_table* table);
/* A batch with an explicit tuning, whatever the context's table holds. */
lp_status lp_batch_create_tuned(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans,
                                uint32_t nscans, const lp_tuning* tuning, lp_batch** out);
lp_status lp_batch_get_tuning(const lp_batch* batch, lp_tuning* out);

typedef struct lp_autotune_report
{
    uint32_t trials;  /* candidate tunings timed (the starting one included) */
    float start_ms;   /* device time per execution of the starting tuning */
    float best_ms;    /* and of the one chosen */
} lp_autotune_report;

/* Coordinate descent over the tuning fields on these scans: each candidate is a prepared batch
 * replayed as a CUDA graph, timed with CUDA events over `iters` executions back to back (no L2 flush
 * between them, as batches follow one another in a stream); a candidate replaces the current choice only if at least 1 % faster. Starts from the
 * table's entry for the scans' bucket (else the defaults) and stores the choice there. trial_ms /
 * trial_cfg (trial_cap entries, either may be null) receive every timed candidate in order. */
lp_status lp_autotune(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans, uint32_t nscans,
                      uint32_t iters, lp_tuning_table* table, lp_tuning* best, lp_autotune_report* report,
                      float* trial_ms, lp_tuning* trial_cfg, uint32_t trial_cap);

/* ------------------------------------------------------------------------------------------ */
/* Serving: scans from several sensors submitted as they arrive, continuous batching.          */
/* No counterpart in the reference (its processor node handles one scan per callback).         */
/* ------------------------------------------------------------------------------------------ */
typedef struct lp_server lp_server;

typedef struct lp_server_config
{
    uint64_t memory_budget_bytes; /* device memory reserved once for in-flight batches: one pool from
                                     which each admitted batch takes exactly its planned bytes; a scan
                                     that does not fit the memory free now waits, one larger than the
                                     whole budget is refused (LP_ERR_CAPACITY) */
    uint32_t max_batch_scans;     /* most scans one batch admits */
    uint32_t slots;               /* batches that can be on the GPU at once (each has its own stream) */
} lp_server_config;

typedef struct lp_server_done
{
    uint64_t tag;
    lp_status status;
    uint32_t batch_scans; /* scans in the batch this one ran in */
    double latency_ms;    /* submission -> results in the caller's buffers */
    double queue_ms;      /* submission -> its batch started */
} lp_server_done;

typedef struct lp_server_stats
{
    uint64_t submitted, completed, failed, batches, scans_in_batches, max_batch_seen, pending;
    uint64_t device_bytes;
    uint64_t memory_waits; /* times the queue's head waited for memory to come back */
} lp_server_stats;

void lp_server_config_default(lp_server_config* cfg);
lp_status lp_server_create(int32_t device, const lp_pipeline_config* cfg, const lp_server_config* scfg,
                           lp_server** out);
/* Queues one scan. The input buffers and `out` (with its buffers) must stay valid until the scan
 * is reported by lp_server_poll; results are written there exactly as lp_process_scan would. */
lp_status lp_server_submit(lp_server* server, const lp_scan_input* scan, lp_scan_output* out, uint64_t tag);
/* hold != 0: submitted scans queue but no new batch starts (running ones finish); 0 resumes. For
 * a burst to be batched as it would arrive at once (and for the admission tests). */
lp_status lp_server_hold(lp_server* server, int32_t hold);
/* Finished scans since the last poll (up to capacity); waits up to wait_us for at least one. */
lp_status lp_server_poll(lp_server* server, lp_server_done* done, uint32_t capacity, uint32_t* n_done,
                         uint32_t wait_us);
lp_status lp_server_stats_get(lp_server* server, lp_server_stats* out);
/* Drains the queue, waits for in-flight batches and releases the server. */
void lp_server_destroy(lp_server* server);

#ifdef __cplusplus
}
#endif

#endif /* LIDAR_GB300_BATCH_H */
