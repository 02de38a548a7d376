/*
 * evoc_gb300.h — C ABI of the GB300 (sm_103a) EVoC hot path.
 *
 * This library replaces two Rust calls of evoc-rs 0.2.7 with CUDA kernels:
 *
 *   build_fuzzy_simplicial_set + coo_to_adjacency_list
 *       (src/graph/fuzzy_graph.rs:275-295 and :242-256,
 *        called at src/lib.rs:254-256 and src/lib.rs:551-553)
 *   evoc_embedding
 *       (src/graph/embedding.rs:48-298,
 *        called at src/lib.rs:302-309, src/lib.rs:603-610 and
 *        src/graph/label_prop.rs:472-479)
 *
 * Conventions
 *   - Every entry point returns EVOC_OK (0) or a negative status code.
 *     evoc_last_error() returns a message for the last failure on a context.
 *   - Host pointers are caller-owned. Output buffers are caller-allocated,
 *     with sizes given by the accompanying counts.
 *   - Graphs and embedding plans are opaque device-resident handles that are
 *     released with their *_free function.
 *   - Calls are synchronous: on return every output has been written.
 *   - A context owns one CUDA stream and must be used by one host thread at a
 *     time. Different contexts are independent.
 *   - Node ids are uint32; n must be below 2^32 - 1. Entry offsets are int64.
 *   - A kNN row shorter than k is padded at its end with index
 *     EVOC_KNN_PAD; padded entries are ignored (their distance is unused).
 *
 * Numerics (f32 throughout, like the reference's GPU stance, README.md:125-129)
 *   - exp() is the library's own Cody-Waite/Taylor exponential (<= 2 ulp).
 *   - Negative samples come from a Philox4x32-10 stream keyed by the seed and
 *     the edge id, not from rand::SmallRng (embedding.rs:173-175, :231).
 *   - Per-node neighbour order is ascending column, not FxHashMap order
 *     (fuzzy_graph.rs:196-205).
 *   - The per-node gradient is summed serially in incidence-list order, each
 *     fired edge's attraction before its negatives, exactly as the
 *     reference's loop (embedding.rs:203-248). Results are bit-reproducible
 *     and do not depend on launch configuration.
 */
#ifndef EVOC_GB300_H
#define EVOC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EVOC_ABI_VERSION 1

#if defined(__GNUC__)
#define EVOC_API __attribute__((visibility("default")))
#else
#define EVOC_API
#endif

/* status codes */
#define EVOC_OK 0
#define EVOC_ERR_INVALID_ARGUMENT (-1) /* bad pointer, size or parameter     */
#define EVOC_ERR_INVALID_INPUT (-2)    /* bad index / value in input arrays  */
#define EVOC_ERR_UNSUPPORTED (-3)      /* valid but outside supported range  */
#define EVOC_ERR_CUDA (-4)             /* CUDA runtime error                 */
#define EVOC_ERR_OUT_OF_MEMORY (-5)    /* device allocation failed           */
#define EVOC_ERR_NO_DEVICE (-6)        /* no usable sm_103 device            */
#define EVOC_ERR_INTERNAL (-7)         /* device-side self-check failed      */

#define EVOC_KNN_PAD 0xFFFFFFFFu

typedef struct evoc_ctx evoc_ctx_t;
typedef struct evoc_graph evoc_graph_t;
typedef struct evoc_plan evoc_plan_t;

/* Mirror of EvocEmbeddingParams (src/graph/mod.rs:22-49; defaults :52-67).
 * The fields n_label_prop_iter, base_init_threshold and scaling are not read
 * by evoc_embedding and are therefore absent. */
typedef struct {
  int32_t n_epochs;           /* default 50   */
  float noise_level;          /* default 0.5  */
  float negative_sample_rate; /* default 1.0  */
  float initial_alpha;        /* default 0.1  */
  float beta1;                /* default 0.5  (UMAP_BETA1, mod.rs:16) */
  float beta2;                /* default 0.9  (UMAP_BETA2, mod.rs:18) */
  float eps;                  /* default 1e-7 */
} evoc_embed_params_t;

/* Per-epoch work counts of an embedding run, from the deterministic
 * epochs-per-sample schedule (embedding.rs:98-118, :274-286). */
typedef struct {
  int64_t fired_edges;   /* undirected edges with epoch_of_next_sample <= t */
  int64_t negatives;     /* negative draws made at epoch t (incl. k == node) */
  int64_t active_nodes;  /* nodes with at least one fired incident edge      */
} evoc_epoch_stats_t;

/* ---- library / context --------------------------------------------------- */

/* ABI version of the loaded library (EVOC_ABI_VERSION). No counterpart. */
EVOC_API int evoc_abi_version(void);

/* Fill *p with the reference defaults (EvocEmbeddingParams::default,
 * src/graph/mod.rs:52-67). */
EVOC_API void evoc_embed_params_default(evoc_embed_params_t* p);

/* Create a context on CUDA device `device`. Replaces the implicit rayon
 * global pool of the reference (no counterpart function). */
EVOC_API int evoc_ctx_create(int device, evoc_ctx_t** out);
/* Graphs and plans created on a context must be freed before the context is
 * destroyed: they release their device memory on its stream. */
EVOC_API void evoc_ctx_destroy(evoc_ctx_t* ctx);

/* Message of the last failure on ctx (never NULL). With ctx == NULL the
 * message of the last failed evoc_ctx_create on this thread is returned. */
EVOC_API const char* evoc_last_error(const evoc_ctx_t* ctx);

/* The context's cudaStream_t (as void*), for callers that enqueue their own
 * work or events around the library's (no counterpart). */
EVOC_API void* evoc_ctx_stream(const evoc_ctx_t* ctx);

/* Bisection steps of the most recent smooth_knn_dist pass on ctx (by
 * evoc_smooth_knn_dist or a fuzzy set): the number of row-sum evaluations
 * over all rows, each of which evaluates one exp per row entry. A work
 * count for measurement (no counterpart). */
EVOC_API int evoc_ctx_smooth_knn_steps(evoc_ctx_t* ctx, int64_t* steps);

/* ---- fuzzy simplicial set ------------------------------------------------ */

/* smooth_knn_dist (src/graph/fuzzy_graph.rs:33-98) on host arrays.
 * dists: n*k row-major; row i has row_len[i] entries (row_len may be NULL:
 * every row has k). k_target is the usize `k` of the reference (target =
 * log2(k_target)). Writes sigmas[n], rhos[n]. */
EVOC_API int evoc_smooth_knn_dist(evoc_ctx_t* ctx, const float* dists,
                         const int32_t* row_len, int64_t n, int32_t k,
                         uint64_t k_target, float local_connectivity,
                         int32_t n_iter, float* sigmas, float* rhos);

/* build_fuzzy_simplicial_set (fuzzy_graph.rs:275-295) followed by
 * coo_to_adjacency_list (fuzzy_graph.rs:242-256), from a host kNN graph.
 * knn_idx/knn_dist: n*k row-major (rows padded with EVOC_KNN_PAD).
 * effective_n_neighbours: the reference's T-valued effective k
 * (lib.rs:253: neighbour_scale * n_neighbours). symmetrise: fuzzy union
 * (fuzzy_graph.rs:174-228) when nonzero. The result stays on the device. */
EVOC_API int evoc_fuzzy_set(evoc_ctx_t* ctx, const uint32_t* knn_idx,
                   const float* knn_dist, int64_t n, int32_t k,
                   float effective_n_neighbours, int symmetrise,
                   evoc_graph_t** out_graph);

/* Same as evoc_fuzzy_set with knn_idx/knn_dist already in device memory of
 * the context's device. Optionally also returns sigmas/rhos (device, n each;
 * NULL to skip). */
EVOC_API int evoc_fuzzy_set_device(evoc_ctx_t* ctx, const uint32_t* d_knn_idx,
                          const float* d_knn_dist, int64_t n, int32_t k,
                          float effective_n_neighbours, int symmetrise,
                          float* d_sigmas, float* d_rhos,
                          evoc_graph_t** out_graph);

/* evoc_fuzzy_set_device on a raw device kNN search result that may include
 * each query itself: n rows of k_raw candidates (for example the k + 1
 * neighbours of a GPU self-query). Row i keeps its first k entries whose
 * index is not i, in order, padding with EVOC_KNN_PAD -- the self removal of
 * nearest_neighbour_gpu.rs:289-300, done on the device so the graph never
 * makes the Vec<Vec<usize>> round trip through the host (lib.rs:218-246).
 * Candidate rows that are padded must be padded at their ends. */
EVOC_API int evoc_fuzzy_set_device_raw(evoc_ctx_t* ctx, const uint32_t* d_knn_idx_raw,
                                       const float* d_knn_dist_raw, int64_t n,
                                       int32_t k_raw, int32_t k,
                                       float effective_n_neighbours, int symmetrise,
                                       evoc_graph_t** out_graph);

/* The fuzzy sets of n_problems independent kNN graphs in one pass: problem q
 * has n_per[q] rows of knn_idx[q] / knn_dist[q] (host, n_per[q] x k, indices
 * local to the problem, EVOC_KNN_PAD padding). The result is one
 * block-diagonal graph whose rows are the problems' rows in order; block q
 * equals evoc_fuzzy_set of problem q alone, with its indices shifted by the
 * sizes of the problems before it. Use it with evoc_plan_create_blocks or
 * evoc_embed_blocks (no counterpart: many clustering problems at once). */
EVOC_API int evoc_fuzzy_set_batched(evoc_ctx_t* ctx, int32_t n_problems,
                                    const uint32_t* const* knn_idx,
                                    const float* const* knn_dist, const int64_t* n_per,
                                    int32_t k, float effective_n_neighbours, int symmetrise,
                                    evoc_graph_t** out_graph);

/* Upload a weighted adjacency list (the reference's Vec<Vec<(usize, T)>>)
 * given as CSR: indptr[n+1], indices[nnz], weights[nnz] on the host. */
EVOC_API int evoc_graph_from_csr(evoc_ctx_t* ctx, const int64_t* indptr,
                        const uint32_t* indices, const float* weights,
                        int64_t n, evoc_graph_t** out_graph);

/* Scratch of evoc_knn_to_csr_noalloc: one device array of this many bytes.
 * CUDA loads the library's device code lazily (the default since CUDA 12.2),
 * so a GPU holds the array from the first evoc_knn_to_csr_noalloc call on it
 * (or from process start with CUDA_MODULE_LOADING=EAGER) until the process
 * exits. */
#define EVOC_NOALLOC_SCRATCH_BYTES (16u << 20)

/* Weighted directed kNN graph without allocating anything (no counterpart in
 * the reference). For callers that must not allocate device memory while
 * they run, such as services that reserve their whole device-memory budget
 * up front, or host frameworks that own the device heap and forbid operators
 * to call cudaMalloc. evoc_fuzzy_set_device allocates its scratch and its
 * result, so those callers cannot use it.
 *
 * Computes exactly what evoc_fuzzy_set_device computes with symmetrise = 0
 * (smooth_knn_dist + knn_to_coo + coo_to_adjacency_list): rows in kNN order,
 * self loops dropped. Inputs d_knn_idx/d_knn_dist (n*k, rows padded with
 * EVOC_KNN_PAD) and outputs d_indptr[n+1], d_indices[capacity] and
 * d_weights[capacity] are caller-owned device memory on the current device;
 * *nnz_out receives the entry count. The work runs on `stream` (a
 * cudaStream_t, NULL for the default stream); the call returns when it is
 * done.
 *
 * Limits and sharing:
 * - Per-row scratch comes from a fixed file-scope device array, so
 *   n <= (EVOC_NOALLOC_SCRATCH_BYTES - 256) / 16 = 1,048,560 rows. Larger n is
 *   rejected with EVOC_ERR_UNSUPPORTED, and a capacity below the entry count
 *   with EVOC_ERR_INVALID_ARGUMENT.
 * - All calls on a device share that array. Calls whose GPU work overlaps
 *   race on it.
 * - The first call on a device loads this code onto the device, which places
 *   the array and the kernels in device memory (about 16 MiB), and looks up
 *   the array's device address. So make a first call (a one-row call will
 *   do) at start-up, before the caller reserves its memory budget and before
 *   any stream capture; or set CUDA_MODULE_LOADING=EAGER before CUDA starts.
 * - The address is kept per device for the life of the process. Do not reset
 *   a device (cudaDeviceReset) while the library is in use on it: later calls
 *   would pass a stale address.
 * - Errors are reported through evoc_last_error(NULL). */
EVOC_API int evoc_knn_to_csr_noalloc(const uint32_t* d_knn_idx,
                                     const float* d_knn_dist, int64_t n,
                                     int32_t k, float effective_n_neighbours,
                                     int64_t* d_indptr, uint32_t* d_indices,
                                     float* d_weights, int64_t capacity,
                                     int64_t* nnz_out, void* stream);

/* Number of nodes and of directed entries of a graph. */
EVOC_API int evoc_graph_info(const evoc_graph_t* g, int64_t* n, int64_t* nnz);

/* Copy a graph to host CSR arrays (indptr[n+1], indices[nnz], weights[nnz]);
 * rows hold the adjacency list of coo_to_adjacency_list in order. */
EVOC_API int evoc_graph_export(const evoc_graph_t* g, int64_t* indptr,
                      uint32_t* indices, float* weights);

EVOC_API void evoc_graph_free(evoc_graph_t* g);

/* ---- node embedding -------------------------------------------------------
 * evoc_embedding (src/graph/embedding.rs:48-298).
 * dim: n_components (1..16). init: host n*dim (row-major) or NULL for the
 * uniform(-0.25, 0.25) initialisation (embedding.rs:69-76). out: host n*dim.
 * verbose follows parse_verbosity_level (prelude.rs:54-61): 2 prints every
 * 10 epochs like embedding.rs:288-291. */
EVOC_API int evoc_embed(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t dim,
               const evoc_embed_params_t* params, const float* init,
               uint64_t seed, int32_t verbose, float* out);

/* A plan holds the per-graph set-up of evoc_embedding (edge extraction,
 * schedule, per-node incidence lists: embedding.rs:78-175) so that the epoch
 * loop (embedding.rs:178-292) can be run repeatedly. */
EVOC_API int evoc_plan_create(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t dim,
                     const evoc_embed_params_t* params, uint64_t seed,
                     evoc_plan_t** out_plan);

/* One plan over n_problems independent graphs (problem q uses seeds[q]): its
 * device rows are the problems' rows concatenated in order, and every epoch
 * is one launch over all of them. Each problem's result equals its own plan's
 * bit for bit. The many coarse embeddings of label_prop.rs:466-479, or many
 * clustering problems, run this way. */
EVOC_API int evoc_plan_create_batched(evoc_ctx_t* ctx, int32_t n_problems,
                                      const evoc_graph_t* const* graphs, int32_t dim,
                                      const evoc_embed_params_t* params,
                                      const uint64_t* seeds, evoc_plan_t** out_plan);

/* evoc_plan_create_batched for the blocks of one block-diagonal graph (as
 * evoc_fuzzy_set_batched makes): block q is rows [sum of n_per[0..q), + n_per[q]),
 * and an edge between two blocks is an error (EVOC_ERR_INVALID_INPUT). */
EVOC_API int evoc_plan_create_blocks(evoc_ctx_t* ctx, const evoc_graph_t* g,
                                     int32_t n_problems, const int64_t* n_per, int32_t dim,
                                     const evoc_embed_params_t* params,
                                     const uint64_t* seeds, evoc_plan_t** out_plan);

/* evoc_embed_batched for the blocks of one block-diagonal graph: outs[q]
 * (host, n_per[q] * dim) receives block q's embedding, which equals
 * evoc_embed of block q alone with seeds[q]; inits is NULL or one host
 * array per block. */
EVOC_API int evoc_embed_blocks(evoc_ctx_t* ctx, const evoc_graph_t* g, int32_t n_problems,
                               const int64_t* n_per, int32_t dim,
                               const evoc_embed_params_t* params, const float* const* inits,
                               const uint64_t* seeds, float* const* outs);

/* Run the epoch loop from d_init (device n*dim, or NULL for the random
 * initialisation) and write d_out (device n*dim). d_init may equal d_out. */
EVOC_API int evoc_plan_run_device(evoc_plan_t* plan, const float* d_init, float* d_out);

/* As evoc_plan_run_device but only enqueues the work on the context's stream
 * and returns without waiting (no counterpart; for callers that overlap or
 * time the loop with their own events on evoc_ctx_stream). */
EVOC_API int evoc_plan_enqueue_device(evoc_plan_t* plan, const float* d_init,
                                      float* d_out);

/* Runs the epoch loop like evoc_plan_run_device, launching each epoch
 * separately with CUDA events between launches, and writes the device time of
 * every epoch launch in milliseconds to epoch_ms[params.n_epochs]
 * (measurement hook, no counterpart). */
EVOC_API int evoc_plan_profile_epochs(evoc_plan_t* plan, const float* d_init,
                                      float* d_out, float* epoch_ms);

/* Measures the L2 random-gather bandwidth for 32-byte rows (one dim-8 f32
 * row, the epoch kernel's source-row gather) over a device buffer of `bytes`
 * (64 MB keeps it L2-resident): *gbs receives gathered GB/s, best of five
 * timed launches after three warm-up launches. Measurement hook for the
 * roofline's L2 bound (no counterpart). */
EVOC_API int evoc_gather_peak(evoc_ctx_t* ctx, int64_t bytes, double* gbs);

/* Epoch-kernel configuration of a plan (no counterpart): variant 0..3 of the
 * gradient-slots kernel as (slot window, slots per lane per group) = (128, 2),
 * (64, 2), (256, 2), (128, 1), launched once per epoch (the epoch loop is
 * captured in a CUDA graph); variants 4..7 the same kernels with all epochs
 * in one persistent cooperative launch, a grid-wide barrier between epochs
 * (a barrier wait that exceeds 2 s ends the launch with EVOC_ERR_INTERNAL);
 * warps (32-node tiles) per thread block 1, 2 or 4; persistent blocks per SM
 * capped at blocks_per_sm (0: as many as fit). Every configuration gives
 * identical results; only speed differs. */
EVOC_API int evoc_plan_set_config(evoc_plan_t* plan, int32_t variant,
                                  int32_t warps_per_block, int32_t blocks_per_sm);

/* Autotuner (no counterpart): times every configuration above on a sample of
 * the plan's epochs (CUDA events on the context's stream) and keeps the
 * fastest. The choice is cached per plan shape (padded dim, node and slot
 * counts on a half-octave grid, one or many problems, epochs, SM count) for
 * the process, and in the file named by the EVOC_TUNE_CACHE environment
 * variable when it is set; a cached shape is configured without timing.
 * The variant found fastest on sampled epochs is also timed over a whole run
 * in both launch forms. config (3 values, may be NULL) receives (variant,
 * warps_per_block, blocks_per_sm); *ms_per_launch (may be NULL) the chosen configuration's
 * time per epoch launch (0 when nothing was tuned: no slots, no edges, or
 * fewer than 2 epochs). */
EVOC_API int evoc_plan_autotune(evoc_plan_t* plan, int32_t* config, float* ms_per_launch);

/* Layout facts of a plan (any pointer may be NULL): undirected edges,
 * per-node incidence entries (2 per edge), negative-count bit planes per
 * epoch, warps (32-node tiles) per thread block of the epoch kernel, and the
 * number of gradient slots over all epochs (one per fired incidence entry and
 * one per negative sample; 0 when the epoch kernel scans the bit planes
 * instead) (no counterpart). */
EVOC_API int evoc_plan_info(const evoc_plan_t* plan, int64_t* n_edges,
                            int64_t* n_incidence, int32_t* neg_planes,
                            int32_t* warps_per_block, int64_t* n_slots);

/* Per-epoch work counts (stats[params.n_epochs]). */
EVOC_API int evoc_plan_stats(const evoc_plan_t* plan, evoc_epoch_stats_t* stats);

/* Debug/parity hook: run epochs [start_epoch, end_epoch) from the host
 * embedding `init` with zero Adam moments, after advancing the schedule
 * through epochs [0, start_epoch) (embedding.rs:274-286 only). Writes the
 * resulting embedding to out (host n*dim) and, if grad_out is not NULL, the
 * gradient of the last epoch run (embedding.rs:187-253) to grad_out
 * (host n*dim; zeros for inactive nodes). */
EVOC_API int evoc_plan_debug_run(evoc_plan_t* plan, const float* init,
                        int32_t start_epoch, int32_t end_epoch, float* out,
                        float* grad_out);

EVOC_API void evoc_plan_free(evoc_plan_t* plan);

/* ---- batched embedding -----------------------------------------------------
 * Many independent evoc_embedding problems in one launch per epoch (no
 * counterpart in the reference). graphs[p], inits[p] (host or NULL),
 * seeds[p], outs[p] (host n_p*dim). All problems share dim and params.
 * Results equal those of separate evoc_embed calls bit for bit. */
EVOC_API int evoc_embed_batched(evoc_ctx_t* ctx, int32_t n_problems,
                       const evoc_graph_t* const* graphs, int32_t dim,
                       const evoc_embed_params_t* params,
                       const float* const* inits, const uint64_t* seeds,
                       float* const* outs);

/* ---- label propagation partition -------------------------------------------
 * label_prop_loop (src/graph/label_prop.rs:202-230), the partition step of
 * label_propagation_init (:537-564): approx_n_parts seed nodes (default
 * clamp(8 sqrt(n), 256, 16384), at most n), n_iter conservative propagation
 * rounds (default 20; :45-92), the sequential mop-up of unlabelled nodes
 * (:105-142) and the remap to 0..n_parts (:155-180). partition (host, n)
 * receives each node's part; *n_parts the number of parts. Vote sums are the
 * reference's f32 additions in row order; the seed and fallback draws come
 * from Philox4x32-10 instead of rand::SmallRng. */
EVOC_API int evoc_label_prop_partition(evoc_ctx_t* ctx, const evoc_graph_t* g,
                                       int64_t approx_n_parts, int32_t n_iter, uint64_t seed,
                                       uint32_t* partition, int64_t* n_parts);

/* build_mst (src/clustering/mst.rs:82-166): Boruvka's minimum spanning tree
 * of n points (row-major n x dim f32, dim 1..16, finite) over mutual
 * reachability distance, the first step of the clustering stage. Core
 * distance = squared distance to the min(min_samples, n - 1)-th nearest
 * other point (min_samples <= 64 after that clamp); edge weight = the square
 * root of max(d^2, core_u, core_v). Ties follow fixed rules where the
 * reference leaves them to its KD-tree's traversal and hash-map order: a
 * point's nearest other-component point is the smallest index among equal
 * values, a component's pick the point with the smallest index among equal
 * values, and each round's picks are added in ascending order of their
 * component's smallest point index. u, v, w (host, n - 1 entries each)
 * receive the edges in insertion order; *n_edges the count (n - 1 for n >= 1
 * and finite distances). */
EVOC_API int evoc_build_mst(evoc_ctx_t* ctx, const float* data, int64_t n, int32_t dim,
                            int32_t min_samples, int64_t* u, int64_t* v, float* w,
                            int64_t* n_edges);

/* The same with device-resident points and outputs. */
EVOC_API int evoc_build_mst_device(evoc_ctx_t* ctx, const float* d_data, int64_t n,
                                   int32_t dim, int32_t min_samples, int64_t* d_u,
                                   int64_t* d_v, float* d_w, int64_t* n_edges);

/* label_propagation_init (src/graph/label_prop.rs:537-564), the initial
 * embedding evoc() computes before the embedding (lib.rs:271-284): recursive
 * coarsening by the label-propagation partition (clamp(8 sqrt(n), 256,
 * 16384) parts at the top, a quarter per level; 20 rounds), coarse graph
 * clip(N^T G B) and coarse data per level, a PCA (data given, dim <= d) or
 * random base case below 64 nodes, a 50-epoch embedding of each coarse graph
 * (initial_alpha 0.05, seed + 4000), and the expansion averaged with the
 * direct term, centred and scaled by 0.1 (:403-535). g is the fuzzy set of
 * the points; data (host, n x d f32) or NULL; out (host, n x dim) receives
 * the initial embedding, for evoc_embed's init. Sums follow the reference's
 * sparse-algebra orders (sparse.rs:256-568); random draws are Philox, and the
 * PCA base case signs each component so its largest entry is positive. */
EVOC_API int evoc_label_propagation_init(evoc_ctx_t* ctx, const evoc_graph_t* g,
                                         int32_t dim, const float* data, int64_t d,
                                         uint64_t seed, float* out);

/* The same with device-resident data (d_data may be NULL) and output. */
EVOC_API int evoc_label_propagation_init_device(evoc_ctx_t* ctx, const evoc_graph_t* g,
                                                int32_t dim, const float* d_data,
                                                int64_t d, uint64_t seed, float* d_out);

/* ---- learned warm start ----------------------------------------------------
 * No counterpart in the reference: a multilayer perceptron
 *   in_dim -> hidden -> GELU -> hidden -> GELU -> out_dim
 * that predicts an initial embedding (the `initial_embedding` argument of
 * evoc_embedding, embedding.rs:48-76) from the input points, so a run needs
 * fewer epochs. BF16 tensor-core GEMMs with FP32 accumulation; FP32 master
 * weights trained by Adam on layouts the plain optimiser produced, each
 * aligned to the current prediction by an orthogonal Procrustes rotation.
 *
 * Parameters are one packed float array of evoc_mlp_n_params() values:
 *   W1 (hidden x in_dim), b1 (hidden), W2 (hidden x hidden), b2 (hidden),
 *   W3 (out_dim x hidden), b3 (out_dim)
 * with weight matrices row-major, output by input.
 * in_dim and hidden are multiples of 8; 1 <= out_dim <= 16. */
typedef struct evoc_mlp evoc_mlp_t;

typedef struct {
  int32_t steps;       /* Adam steps                                  (3000)  */
  int32_t batch;       /* rows per step, drawn with replacement       (8192)  */
  int32_t align_every; /* steps between Procrustes re-alignments      (250)   */
  int32_t align_rows;  /* rows per instance that fix the rotation     (65536) */
  float lr;            /* Adam step size                              (1e-3)  */
  float beta1;         /*                                             (0.9)   */
  float beta2;         /*                                             (0.999) */
  float eps;           /*                                             (1e-8)  */
  float lr_end;        /* step size reached linearly at the last step (1e-4)  */
  uint64_t seed;       /* row sampling                                (0)     */
} evoc_mlp_train_params_t;

EVOC_API void evoc_mlp_train_params_default(evoc_mlp_train_params_t* p);

/* Create a network with seeded Linear-layer initialisation (uniform in
 * +-1/sqrt(fan_in)). Free it before destroying its context. */
EVOC_API int evoc_mlp_create(evoc_ctx_t* ctx, int32_t in_dim, int32_t hidden,
                             int32_t out_dim, uint64_t seed, evoc_mlp_t** out);
EVOC_API void evoc_mlp_free(evoc_mlp_t* mlp);
EVOC_API int64_t evoc_mlp_n_params(const evoc_mlp_t* mlp);

/* FP32 master parameters, packed as above (host arrays of n_params).
 * evoc_mlp_set_params also resets the Adam state. */
EVOC_API int evoc_mlp_get_params(const evoc_mlp_t* mlp, float* params);
EVOC_API int evoc_mlp_set_params(evoc_mlp_t* mlp, const float* params);

/* Predict out (n x out_dim) from points x (n x in_dim): host f32 buffers, or
 * device buffers with BF16 points (16-byte aligned) and f32 output. */
EVOC_API int evoc_mlp_predict(evoc_mlp_t* mlp, const float* x, int64_t n, float* out);
EVOC_API int evoc_mlp_predict_device(evoc_mlp_t* mlp, const uint16_t* d_x_bf16,
                                     int64_t n, float* d_out);

/* Parity hook: the mean squared error of the prediction against target
 * (n x out_dim) and its gradient for every parameter (packed as above), for
 * host points x (n x in_dim, rounded to BF16). Does not update the network. */
EVOC_API int evoc_mlp_gradients(evoc_mlp_t* mlp, const float* x, const float* target,
                                int64_t n, float* loss, float* grad);

/* Train on n_instances (points, layout) pairs in device memory: d_x_bf16[i]
 * (n_rows[i] x in_dim BF16, 16-byte aligned) and d_layouts[i]
 * (n_rows[i] x out_dim f32, e.g. evoc_embed output). loss_history (host,
 * params->steps floats, or NULL) receives each step's mean squared error. */
EVOC_API int evoc_mlp_fit_device(evoc_mlp_t* mlp, int32_t n_instances,
                                 const uint16_t* const* d_x_bf16,
                                 const float* const* d_layouts, const int64_t* n_rows,
                                 const evoc_mlp_train_params_t* params,
                                 float* loss_history);

/* Round count f32 values to BF16 (nearest even) on the device. */
EVOC_API int evoc_to_bf16_device(evoc_ctx_t* ctx, const float* d_in, int64_t count,
                                 uint16_t* d_out);

/* Self-test of the bounded-wait path of the tcgen05 kernels: launches a
 * kernel that waits on an mbarrier nothing arrives on, for limit_ms
 * (1..2000), and returns the resulting EVOC_ERR_INTERNAL ("timed out"). The
 * context stays usable. No counterpart. */
EVOC_API int evoc_selftest_wait_timeout(evoc_ctx_t* ctx, int32_t limit_ms);

/* Host only: the orthogonal d x d matrix R maximising trace(R^T M) for a
 * row-major d x d M (R = U V^T for M = U S V^T), 1 <= d <= 16. With
 * M = X^T Y for centred X and Y, X R is the rotation of X closest to Y. */
EVOC_API int evoc_procrustes(const double* m, int32_t d, double* r);

#ifdef __cplusplus
}
#endif

#endif /* EVOC_GB300_H */
