/*
 * hashdag_gpu.h -- C ABI of the GB300 HashDAG edit engine.
 *
 * The engine keeps a HashDAG node pool resident in device memory and applies
 * stateless geometry edits to it with sm_103a kernels.  The pool keeps the
 * reference's storage format word for word:
 *   - a NodePointer is a global word index into a bucketed, paged address space,
 *     0xFFFFFFFF is Null (include/hashdag/NodePointer.hpp:13-31);
 *   - an inner node is a mask word (low 8 bits = child mask) followed by the
 *     non-null children in ascending child order; a leaf is two words holding
 *     a 4x4x4 bitmask (include/hashdag/NodePool.hpp:214-317);
 *   - a node lives in bucket  base[level] + (hash(node) & (buckets_at_level-1))
 *     and never straddles a page; the tail of a page that cannot hold the next
 *     node is zero-filled (include/hashdag/NodePool.hpp:134-212);
 *   - hash = MurmurHash3-x86-32 body (seed 0, length in words) for inner nodes
 *     and the 64-bit finaliser truncated to 32 bits for leaves
 *     (include/hashdag/Hasher.hpp:21-48).
 * So a pool downloaded with hd_pool_read_* can be handed to the reference's
 * CPU NodePoolBase / NodePoolTraversal unchanged, and a pool built by the
 * reference can be uploaded with hd_pool_upload.
 *
 * All entry points return an hd_status.  None falls back silently: where the
 * reference returns the stale node when a bucket is full
 * (include/hashdag/NodePool.hpp:138-139,195,210) this library returns
 * HD_ERR_BUCKET_FULL and leaves *out_root equal to the input root.
 * Calls on one pool are serialised by an internal mutex; different pools may
 * be used from different threads and streams at the same time.
 */
#ifndef HASHDAG_GPU_H
#define HASHDAG_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hd_status {
	HD_OK = 0,
	HD_ERR_INVALID_ARG = 1,  /* bad config / argument (reference: Config::Validate false, Create -> nullptr) */
	HD_ERR_BUCKET_FULL = 2,  /* a node did not fit into its bucket (reference: silent fallback) */
	HD_ERR_POOL_OOM = 3,     /* the device page heap has no free page left */
	HD_ERR_INDEX_FULL = 4,   /* the device dedup index has no free slot left */
	HD_ERR_CAPACITY = 5,     /* edit workspace too small (hd_edit grows it and retries by itself) */
	HD_ERR_CUDA = 6,         /* a CUDA runtime call failed */
	HD_ERR_TIMEOUT = 7,      /* a bounded device-side wait ran out */
	HD_ERR_NO_DEVICE = 8,    /* no CUDA device / extension not usable */
	HD_ERR_INTERNAL = 9,     /* a device-side consistency check failed (work skipped, nothing corrupted) */
} hd_status;

#define HD_NULL_PTR 0xFFFFFFFFu
#define HD_MAX_LEVELS 24

/* WordSpanHasher choice (include/hashdag/NodePool.hpp:23, include/hashdag/Hasher.hpp:21-48).
 * HD_HASHER_ZERO maps every node to the first bucket of its level, like the
 * reference test fixture ZeroHasher (test/test.cpp:10-12). */
typedef enum hd_hasher { HD_HASHER_MURMUR32 = 0, HD_HASHER_ZERO = 1 } hd_hasher;

/* hashdag::Config<uint32_t> (include/hashdag/Config.hpp:15-57).
 * node_levels = bucket_bits_each_level.size(); resolution = 2^(node_levels+1). */
typedef struct hd_config {
	uint32_t word_bits_per_page;
	uint32_t page_bits_per_bucket;
	uint32_t node_levels;
	uint32_t hasher; /* hd_hasher */
	uint32_t bucket_bits_each_level[HD_MAX_LEVELS];
} hd_config;

/* Stateless editors of the reference application (src/main.cpp:32-150).
 *   SPHERE: voxel p is inside iff |p - center|^2 <= r2 (integer voxel corner).
 *   AABB:   voxel p is inside iff p0 <= p < p1 on every axis (half-open box).
 * FILL sets the voxels inside, DIG clears them (SphereEditor<kFill/kDig>;
 * the AABB dig follows the same pattern).  A list of edits is applied in
 * order: per voxel the last edit whose shape covers it decides. */
typedef enum hd_shape { HD_SHAPE_SPHERE = 0, HD_SHAPE_AABB = 1 } hd_shape;
/* HD_OP_PAINT: colour edits only (hd_vbr_edit): recolour without changing the geometry */
typedef enum hd_op { HD_OP_FILL = 0, HD_OP_DIG = 1, HD_OP_PAINT = 2 } hd_op;

typedef struct hd_edit_desc {
	uint32_t shape;  /* hd_shape */
	uint32_t op;     /* hd_op */
	uint32_t p0[3];  /* sphere centre, or box min (inclusive), voxel units */
	uint32_t p1[3];  /* box max (exclusive); ignored for spheres */
	uint64_t r2;     /* sphere radius squared; ignored for boxes */
} hd_edit_desc;      /* 40 bytes */

typedef struct hd_pool hd_pool;

typedef struct hd_pool_stats {
	uint64_t heap_pages;       /* physical pages in the device heap */
	uint64_t used_pages;       /* physical pages handed out */
	uint64_t total_buckets;
	uint64_t total_pages;      /* virtual pages (Config::GetTotalPages) */
	uint64_t index_slots;
	uint64_t index_used;       /* dedup index slots holding a node */
	uint32_t max_bucket_words; /* fullest bucket */
	uint32_t words_per_bucket;
} hd_pool_stats;

/* Ray hit of the read path (shader/src/trace.frag:69-270 DAG_RayMarch without LOD).
 * hit = 0 means the ray left the volume.  voxel = integer voxel coordinate of
 * the hit cell's minimum corner, size = its edge in voxels (1 for a voxel),
 * level = voxel_level - log2(size); t = ray parameter at the entry point;
 * pos = hit position in [0,1]^3 as NodePoolTraversal::Traversal returns it
 * (include/hashdag/NodePoolTraversal.hpp:253-255). */
typedef struct hd_hit {
	uint32_t voxel[3];
	uint32_t size;
	uint32_t level;
	uint32_t hit;
	float t;
	float pos[3];
} hd_hit; /* 40 bytes */

/* Pinhole camera (src/Camera.hpp:36-52, shader/src/trace.frag:366-370):
 * ray(u,v) = normalize(look - side*(2u-1) - up*(2v-1)), origin = position,
 * all in [0,1]^3 scene units; u = (px+0.5)/width, v = (py+0.5)/height. */
typedef struct hd_camera {
	float position[3];
	float look[3];
	float side[3];
	float up[3];
} hd_camera;

/* ---- pool lifecycle -------------------------------------------------------
 * replaces NodePoolBase(Config) (include/hashdag/NodePool.hpp:400-403) and
 * DAGNodePool::Create (src/DAGNodePool.cpp:9-47).  heap_pages = device pages
 * reserved for node storage (memory = heap_pages << word_bits_per_page words);
 * index_log2 = log2 of dedup index slots (0 = sized from heap_pages).
 * The filled node of every level (make_filled_node_pointers,
 * include/hashdag/NodePool.hpp:240-262) is inserted at creation. */
hd_status hd_pool_create(const hd_config *config, uint64_t heap_pages, uint32_t index_log2, int device,
                         hd_pool **out_pool);
void hd_pool_destroy(hd_pool *pool);
/* Config::Validate (include/hashdag/Config.hpp:48-56). */
int hd_config_validate(const hd_config *config);
/* DefaultConfig<uint32_t>{...}() (include/hashdag/Config.hpp:59-75). */
void hd_config_default(uint32_t level_count, uint32_t top_level_count, uint32_t word_bits_per_page,
                       uint32_t page_bits_per_bucket, uint32_t bucket_bits_per_top_level,
                       uint32_t bucket_bits_per_bottom_level, hd_config *out);
/* m_filled_node_pointers (include/hashdag/NodePool.hpp:54), one per level. */
hd_status hd_pool_filled_pointers(const hd_pool *pool, uint32_t *out_levels);
hd_status hd_pool_get_stats(const hd_pool *pool, hd_pool_stats *out);
/* Sticky device error word of the pool (for the *_async entry points); 0 = none.
 * hd_pool_clear_error resets it. */
hd_status hd_pool_get_error(const hd_pool *pool, uint32_t *out_error);
hd_status hd_pool_clear_error(hd_pool *pool);

/* ---- edit path ------------------------------------------------------------
 * replaces NodePoolBase::Edit (include/hashdag/NodePool.hpp:405-417) and
 * NodePoolThreadedEdit::ThreadedEdit (include/hashdag/NodePoolThreadedEdit.hpp:104-126)
 * for the stateless editors (include/hashdag/Editor.hpp:36-55, src/main.cpp:32-150).
 * Applies edits[0..n) in order to root and returns the new root.  n = 1 is the
 * plain one-edit form; n > 1 is one level-synchronous batched pass whose
 * voxel result equals applying the edits one after another.  Host edit array;
 * blocks until the result is known.  stream = cudaStream_t or NULL. */
hd_status hd_edit(hd_pool *pool, uint32_t root, const hd_edit_desc *edits, uint32_t n, uint32_t *out_root,
                  void *stream);
/* Same work with device-resident inputs and output and no host synchronisation:
 * d_edits and d_out_root are device pointers; status is reported through the
 * pool's sticky error word (hd_pool_get_error).  The workspace must have been
 * sized by hd_edit_reserve (or a previous hd_edit of at least this size). */
hd_status hd_edit_async(hd_pool *pool, uint32_t root, const hd_edit_desc *d_edits, uint32_t n,
                        uint32_t *d_out_root, void *stream);
/* Same as hd_edit_async but the root is read from device memory (d_root), so a
 * chain of edits can run without any host round trip. */
hd_status hd_edit_async_droot(hd_pool *pool, const uint32_t *d_root, const hd_edit_desc *d_edits, uint32_t n,
                              uint32_t *d_out_root, void *stream);
/* hd_edit_async_droot for a caller that also holds the edits on the host:
 * h_edits (the same n edits, host memory, read before the call returns) sizes
 * the launch the way hd_edit does -- grids from the edits' bounding boxes, and
 * a small pass as one CTA -- while the kernels read d_edits.  Same entry point
 * as the reference's Edit (include/hashdag/NodePool.hpp:405-417) for an edit
 * loop that keeps its root on the device. */
hd_status hd_edit_async_droot_hinted(hd_pool *pool, const uint32_t *d_root, const hd_edit_desc *d_edits,
                                     const hd_edit_desc *h_edits, uint32_t n, uint32_t *d_out_root, void *stream);
/* Size the edit workspace for batches of up to max_edits touching up to
 * max_items nodes per batch and max_list_entries (node, edit) pairs. */
hd_status hd_edit_reserve(hd_pool *pool, uint64_t max_items, uint64_t max_list_entries, uint32_t max_edits);
/* Per-level counters of the last edit pass (arrays of node_levels entries,
 * any may be NULL): items = nodes visited (frontier size), candidates = nodes
 * that went through the dedup pass and their words, inserted = nodes newly
 * appended to buckets and their words.  For diagnosis, the environment
 * variable HD_DEBUG_SYNC (any value) makes every pass launch its kernels
 * directly (no graph), synchronise after each phase and print the pass
 * counters to stderr; the results are the same. */
hd_status hd_edit_last_counters(hd_pool *pool, uint64_t *items, uint64_t *candidates, uint64_t *candidate_words,
                                uint64_t *inserted, uint64_t *inserted_words);
/* Dedup-index statistics of the last edit pass (any may be NULL): index slots
 * visited by all find-or-insert probes, the longest single probe, and failed
 * compare-and-swap attempts on bucket word counts (contention). */
hd_status hd_edit_last_probe_stats(hd_pool *pool, uint64_t *probe_steps, uint64_t *max_probe, uint64_t *cas_retries);
/* Work of the last pass's level-(L-2) leaf kernels (no reference counterpart:
 * the numerator of that phase's roofline): out[0] level-(L-2) nodes rebuilt,
 * out[1] (node, edit) pairs of their edit lists, out[2] base-node words read,
 * out[3] old leaves read from the heap, out[4] read-only lookups of changed
 * leaves, out[5] of these answered by the pass's leaf-pattern cache, out[6]
 * read-only index lookups of level-(L-2) nodes whose children were all known. */
hd_status hd_edit_last_leaf_work(hd_pool *pool, uint64_t *out);
/* Launch shape of the batched pass: grid caps in blocks per SM for each kernel
 * family and the edit-list length above which a node is expanded by a block
 * (level L-2: a warp) instead of a thread.  Results never depend on them. */
typedef struct hd_tuning {
	uint32_t expand_blocks_per_sm;     /* k_expand_short (default 8) */
	uint32_t leaf_blocks_per_sm;       /* k_leafparent_compact / k_leafparent_short (default 12) */
	uint32_t dedup_blocks_per_sm;      /* k_dedup (default 32) */
	uint32_t long_blocks_per_sm;       /* k_expand_long / k_leafparent_long (default 4) */
	uint32_t long_threshold;           /* default 16, at least 1 */
	uint32_t leaf_compact;             /* level-(L-2) leaves: 1 = a warp's deferred leaves (partly covered ones)
	                                      compacted onto all its lanes (k_leafparent_compact, default),
	                                      0 = thread per node (k_leafparent_short) */
} hd_tuning;
hd_status hd_edit_get_tuning(const hd_pool *pool, hd_tuning *out);
hd_status hd_edit_set_tuning(hd_pool *pool, const hd_tuning *tuning);
/* Autotuner: times the batched pass of edits[0..n) on root (the pool is rolled
 * back after every trial, so it ends unchanged) for candidate launch shapes,
 * one parameter at a time, keeps the fastest and installs it.  out (may be
 * NULL) receives the chosen shape; ms_before / ms_after (may be NULL) the
 * device time of the pass with the shape before and after. */
hd_status hd_edit_autotune(hd_pool *pool, uint32_t root, const hd_edit_desc *edits, uint32_t n, hd_tuning *out,
                           float *ms_before, float *ms_after);

/* Checkpoint / rollback of the whole pool state (bucket word counts, page
 * table, heap and index counters, dedup index), kept in device memory.
 * Rollback (stream-ordered) forgets every node inserted after the checkpoint;
 * roots created after it become invalid.  Words past a bucket's word count in
 * reused pages keep stale values (no scan ever reads them). */
hd_status hd_pool_checkpoint(hd_pool *pool);
hd_status hd_pool_rollback(hd_pool *pool, void *stream);
/* Phase timing of edit passes with CUDA events recorded on the pass's own
 * stream: after hd_edit_profile_begin, the next max_passes passes record
 * events; hd_edit_profile_end waits for them and writes, summed over those
 * passes, node_levels+3 phase durations in ms: [0] root+expand (all levels),
 * [1] leaf voxels, then the dedup launch of level L-1 down to 0; [last] finish. */
hd_status hd_edit_profile_begin(hd_pool *pool, uint32_t max_passes);
hd_status hd_edit_profile_end(hd_pool *pool, float *out_ms, uint32_t *out_passes);
/* Kernels this pool has launched since creation. */
uint64_t hd_pool_kernel_launches(const hd_pool *pool);

/* ---- upsert (find-or-insert) ---------------------------------------------
 * replaces upsert_inner_node / upsert_leaf (include/hashdag/NodePool.hpp:159-238).
 * words = n packed nodes back to back (host), lens[i] = word count of node i
 * (2 for a leaf at level node_levels-1, 1+popcount(mask) otherwise).  All
 * nodes go to `level`.  out_ptrs[i] = pointer of the stored or found node. */
hd_status hd_upsert(hd_pool *pool, uint32_t level, const uint32_t *words, const uint32_t *lens, uint32_t n,
                    uint32_t *out_ptrs);

/* Find-or-insert without any allocation (no counterpart in the reference).
 * For callers that cannot call cudaMalloc when they insert nodes -- e.g. an
 * application that gives all device memory to its own allocator up front, or
 * an edit loop that must not take the device synchronisation a cudaMalloc /
 * cudaFree can cause.  Same result as hd_upsert, but device inputs and
 * outputs, stream-ordered, no host synchronisation, and the per-node scratch
 * in a static device array of the library (about 4.7 MB: 224 counters of 8
 * bytes plus 18 words per node for 65536 nodes, held by every GPU that loads
 * the library until the process exits) instead of the pool's workspace.
 * d_nodes: n nodes on the device, 8 child pointers each (Null = 0xFFFFFFFF,
 * child order) below the leaf level, 2 words each at the leaf level.
 * d_out_ptrs: n pointers (device).  At most 65536 nodes per call; larger n
 * returns HD_ERR_INVALID_ARG without running anything.  Failures inside the
 * kernels go to the pool's sticky error (hd_pool_get_error), and then every
 * d_out_ptrs entry of the call is Null: an inner node whose 8 children are all
 * Null (which hd_upsert rejects on the host) sets HD_ERR_INVALID_ARG there,
 * as does any other failure of the call.  A leaf of two zero words is stored
 * like any other leaf, as the reference's upsert_leaf does (edits never
 * produce one: an emptied leaf becomes Null).  The
 * first call on a device looks up the array's device address (make it before
 * any stream capture).  All calls on a device share the one array: calls that
 * overlap on the GPU race. */
hd_status hd_upsert_noalloc(hd_pool *pool, uint32_t level, const uint32_t *d_nodes, uint32_t n, uint32_t *d_out_ptrs,
                            void *stream);

/* ---- host mirror (reference storage hooks) --------------------------------
 * GetBucketRefWords / ReadPage (include/hashdag/NodePool.hpp:22-29,
 * src/DAGNodePool.hpp:56-69).  Virtual page ids are the reference's page ids
 * (bucket << page_bits_per_bucket | page in bucket). */
hd_status hd_pool_read_bucket_words(const hd_pool *pool, uint32_t first_bucket, uint32_t count, uint32_t *out);
/* out[i] = 1 if virtual page i holds data, else 0 (count = total pages). */
hd_status hd_pool_read_page_map(const hd_pool *pool, uint8_t *out);
/* Copies virtual pages page_ids[0..n) to out (n << word_bits_per_page words). */
hd_status hd_pool_read_pages(const hd_pool *pool, const uint32_t *page_ids, uint32_t n, uint32_t *out);
/* Replaces the pool contents with a host pool (e.g. one the reference built):
 * bucket words for every bucket, n pages with their ids and words, and the
 * filled-node pointer per level (NULL = recompute).  Rebuilds the dedup index. */
hd_status hd_pool_upload(hd_pool *pool, const uint32_t *bucket_words, const uint32_t *page_ids, uint32_t n_pages,
                         const uint32_t *page_words, const uint32_t *filled_levels);
/* Generation of the pool's committed words, for incremental host mirrors (the
 * dirty page ranges of src/DAGNodePool.hpp:62-69): every call that rewrites or
 * drops words already in the pool (hd_gc, hd_pool_rollback, hd_pool_upload)
 * increments it.  Between two calls that read the same epoch the pool only
 * appended words: bucket b's new words are [old count, new count) of
 * hd_pool_read_bucket_words, on the pages that range covers. */
hd_status hd_pool_epoch(const hd_pool *pool, uint64_t *out);

/* ---- garbage collection -----------------------------------------------------
 * NodePoolThreadedGC::ThreadedGC (include/hashdag/NodePoolThreadedGC.hpp:29-403):
 * keeps the nodes reachable from roots[0..n_roots) and from the filled nodes,
 * compacts every level into the layout the reference's collector writes with
 * one worker (buckets re-filled in old-pointer order, inner nodes re-hashed
 * into their new buckets), frees every page it no longer needs, rebuilds the
 * dedup index and re-finds the filled nodes.  roots are remapped in place
 * (HD_NULL_PTR stays).  Every root made before the call and not passed in
 * becomes invalid.  Nothing is changed when it fails (a root that is not a
 * level-0 node: HD_ERR_INVALID_ARG; a bucket that cannot hold the nodes that
 * hash to it after compaction: HD_ERR_BUCKET_FULL; not enough device memory
 * for the collection's scratch: HD_ERR_POOL_OOM).  stats may be NULL. */
typedef struct hd_gc_stats {
	uint64_t live_nodes;     /* nodes kept */
	uint64_t words_before;   /* sum of bucket word counts before / after */
	uint64_t words_after;
	uint64_t pages_before;   /* heap pages in use before / after */
	uint64_t pages_after;
} hd_gc_stats;
hd_status hd_gc(hd_pool *pool, uint32_t *roots, uint32_t n_roots, hd_gc_stats *stats);

/* ---- read path --------------------------------------------------------------
 * Point occupancy: out[i] = voxel (xyz[3i], xyz[3i+1], xyz[3i+2]) set under root. */
hd_status hd_query(hd_pool *pool, uint32_t root, const uint32_t *xyz, uint32_t n, uint8_t *out, void *stream);
/* NodePoolTraversal::Traversal<float> (include/hashdag/NodePoolTraversal.hpp:93-256)
 * over n rays: origins/dirs = 3n floats (host), out = n hits (host). */
hd_status hd_trace(hd_pool *pool, uint32_t root, const float *origins, const float *dirs, uint32_t n, hd_hit *out,
                   void *stream);
/* Primary rays of n_cameras pinhole cameras at width x height, device output
 * (d_out = device pointer to n_cameras*width*height hits, camera-major,
 * row-major).  d_counters (device, 3 x u64, may be NULL) accumulates traversal
 * loop iterations, node words read and hits.  Async on stream. */
hd_status hd_trace_pinhole_async(hd_pool *pool, uint32_t root, const hd_camera *cameras, uint32_t n_cameras,
                                 uint32_t width, uint32_t height, hd_hit *d_out, uint64_t *d_counters, void *stream);
/* The same rays and the same hit records (bit for bit, same positions) from
 * the stackless warp-coherent kernel: no per-ray parent stack (the nodes of
 * the last four pushed scales in registers; a pop past them re-descends from
 * the root along the cell's position bits, which arrives at the node the
 * reference's stack holds, NodePoolTraversal.hpp:151-243), and every warp on
 * an 8 x 4 pixel tile.  The node-word counter includes the re-descents. */
hd_status hd_trace_pinhole_stackless_async(hd_pool *pool, uint32_t root, const hd_camera *cameras,
                                           uint32_t n_cameras, uint32_t width, uint32_t height, hd_hit *d_out,
                                           uint64_t *d_counters, void *stream);

/* ---- serving loop ------------------------------------------------------------
 * Several resident scenes (one hd_pool each, all on one device) served from
 * one request stream.  Generalises the reference application's edit loop
 * (src/main.cpp:280-296: one edit at a time on a worker thread while frames
 * trace the last finished root; an edit arriving while another runs is dropped
 * there):
 *   - edit requests of a scene queue in arrival order; whenever the scene's
 *     previous pass has finished, everything queued (up to max_pass_edits
 *     edits) is merged into ONE batched pass (continuous batching);
 *   - admission by free pages: a request is taken into a pass only while the
 *     pages its edits are expected to need (a running per-scene average of
 *     pages per edit) fit into the scene's free heap pages; a request that
 *     does not fit even alone is refused with HD_ERR_POOL_OOM, admitted = 0;
 *   - camera (ray) requests run on ray_slots high-priority streams, each traced
 *     against its scene's last finished root at the moment it starts, so ray
 *     work overlaps the scenes' edit passes on the device;
 *   - a merged pass that fails is re-run request by request from the pass's
 *     input root, so every request gets the status it would get alone;
 *   - with gc_free_fraction set, a scene whose heap runs low is collected
 *     between two of its passes (its ray requests wait meanwhile), so memory
 *     frees up and later requests are admitted again.
 * Results: a merged pass's voxels equal applying its requests one after
 * another (the batched-pass contract of hd_edit); a ray request's hits equal
 * hd_trace_pinhole_async on the recorded root. */
typedef struct hd_server hd_server;

typedef struct hd_server_config {
	uint32_t max_pass_edits;        /* edits merged into one pass at most (0 = 16384) */
	uint32_t ray_slots;             /* concurrent ray requests (0 = 4) */
	uint32_t max_rays_per_request;  /* larger camera requests are refused (0 = 1 << 24) */
	uint32_t reserve_pages;         /* heap pages kept free by admission (0 = heap/64) */
	double pages_per_edit_hint;     /* admission estimate before the first pass (0 = 1.0) */
	double gc_free_fraction;        /* collect a scene (hd_gc, its current root kept) after a pass
	                                   that leaves fewer than this fraction of its heap pages free;
	                                   0 = never */
} hd_server_config;

typedef enum hd_request_kind { HD_REQ_EDIT = 0, HD_REQ_CAMERA = 1 } hd_request_kind;

typedef struct hd_request_result {
	uint64_t id;
	uint32_t kind;           /* hd_request_kind */
	uint32_t scene;
	int32_t status;          /* hd_status of this request */
	uint32_t admitted;       /* 0: refused by admission control (nothing ran) */
	uint32_t root_in;        /* edit: root the pass started from; camera: root traced */
	uint32_t root;           /* edit: scene root after the pass carrying it; camera: root traced */
	uint64_t pass_id;        /* edit: per-scene pass number (requests of one pass share it) */
	uint32_t pass_requests;  /* edit: requests merged into that pass (1 = alone) */
	uint32_t pass_edits;     /* edit: edits in that pass */
	uint64_t rays;           /* camera: rays traced */
	uint64_t hits, steps, node_words; /* camera: traversal counters */
	double t_submit_ms, t_start_ms, t_done_ms; /* ms since hd_server_create */
	uint64_t gc_epoch;       /* collections of the scene before root_in / root were taken: roots
	                            of an older epoch are no longer valid */
} hd_request_result;

typedef struct hd_server_stats {
	uint64_t edit_requests, camera_requests; /* completed */
	uint64_t refused, failed;                /* refused by admission / finished with an error */
	uint64_t edit_passes, edits_applied, rays_traced;
	uint32_t max_pass_requests, queued;      /* largest merge; requests not finished yet */
	double edit_p50_ms, edit_p99_ms, camera_p50_ms, camera_p99_ms; /* submit -> done */
	uint64_t gc_runs;                        /* collections run by the server */
	double gc_ms;                            /* their total wall time */
} hd_server_stats;

/* pools[i] with its current root roots[i] (HD_NULL_PTR = empty) is scene i.
 * The server does not own the pools; it must be destroyed before them, and
 * nothing else may edit, roll back or upload to them while it runs. */
hd_status hd_server_create(hd_pool *const *pools, const uint32_t *roots, uint32_t n_scenes,
                           const hd_server_config *config, hd_server **out_server);
/* Waits for every submitted request, stops the worker threads, frees the
 * server's buffers.  Results not yet retrieved are dropped. */
void hd_server_destroy(hd_server *server);
/* Queues edits[0..n) (host array, copied) for scene; *out_id names the request. */
hd_status hd_server_submit_edits(hd_server *server, uint32_t scene, const hd_edit_desc *edits, uint32_t n,
                                 uint64_t *out_id);
/* Queues n_cameras pinhole cameras at width x height for scene.  host_out
 * (n_cameras*width*height hits, camera-major; pinned memory is fastest) receives
 * the hits and must stay valid until the request is retrieved; NULL keeps
 * them on the device (only the counters are returned). */
hd_status hd_server_submit_camera(hd_server *server, uint32_t scene, const hd_camera *cameras, uint32_t n_cameras,
                                  uint32_t width, uint32_t height, hd_hit *host_out, uint64_t *out_id);
/* Waits up to timeout_ms (< 0: forever) for request id and hands out its
 * result once (HD_ERR_TIMEOUT: not finished yet; HD_ERR_INVALID_ARG: unknown
 * or already retrieved id). */
hd_status hd_server_wait(hd_server *server, uint64_t id, double timeout_ms, hd_request_result *out);
/* paused != 0: no new edit pass and no new ray request starts (running ones
 * finish; submissions keep queueing), e.g. to take a consistent snapshot of
 * the pools.  paused = 0 resumes; queued edits of a scene then merge. */
hd_status hd_server_pause(hd_server *server, int paused);
/* Waits until every request submitted so far has finished
 * (HD_ERR_INVALID_ARG while paused with requests queued). */
hd_status hd_server_drain(hd_server *server);
/* Last finished root of a scene. */
hd_status hd_server_scene_root(hd_server *server, uint32_t scene, uint32_t *out_root);
hd_status hd_server_get_stats(hd_server *server, hd_server_stats *out);

/* Level of detail and the beam prepass of the renderer (shader/src/trace.frag
 * with BEAM_OPTIMIZATION, shader/src/beam.frag, src/rg/BeamPass.cpp):
 *   - descent stops at a cube whose size times proj_factor is below its entry t
 *     (trace.frag:148), so distant geometry is hit at coarser voxels (hd_hit.size);
 *   - beam_proj_factor > 0 first traces one ray per 8x8 pixel block with that
 *     factor and stores t - cube size (+inf on a miss); each pixel then starts at
 *     o + b * d with b = 0.98 * the minimum of the 2x2 block values around it
 *     (the linear MIN-reduction sampler of src/rg/TracePass.cpp:37-54) and uses b
 *     as projection bias; a pixel whose b is +inf is a miss without tracing.
 * proj_factor / beam_proj_factor: hd_projection_factor(fov_y, height, 1 or 8). */
hd_status hd_trace_pinhole_lod_async(hd_pool *pool, uint32_t root, const hd_camera *cameras, uint32_t n_cameras,
                                     uint32_t width, uint32_t height, float proj_factor, float beam_proj_factor,
                                     hd_hit *d_out, uint64_t *d_counters, void *stream);
/* inv_2tan_half_fov / screen_tolerance of src/rg/TracePass.cpp:114-118 (divisor 1)
 * and src/rg/BeamPass.cpp:90-94 (divisor 8), in float like the reference. */
float hd_projection_factor(float fov_y, uint32_t height, uint32_t divisor);

/* ---- workload helpers ------------------------------------------------------
 * Number of grid voxels inside each edit's shape clipped to [0,resolution)^3,
 * summed over the edits (the voxel-edits unit of the benchmark). */
uint64_t hd_count_voxel_edits(const hd_edit_desc *edits, uint32_t n, uint32_t resolution);

/* ---- colour (VBR) ----------------------------------------------------------
 * replaces the application's colour octree DAGColorPool
 * (src/DAGColorPool.hpp:20-218) and colour editing through
 * hashdag::VBREditorWrapper (include/hashdag/VBREditor.hpp:26-107, the chunk
 * writer of include/hashdag/VBRColor.hpp:367-488) driven as the application
 * does (src/main.cpp:224-242), plus the colour lookup of trace.frag:272-356.
 * Octree pointers: 2-bit tag (0 node, 1 colour, 2 leaf, 3 null) over 30 bits
 * of data; the words read back by hd_color_pool_read are the ones the
 * reference's single-threaded NodePoolBase::Edit writes for the same edits. */
#define HD_COLOR_NULL 0xC0000000u
typedef struct hd_color_config {
	uint32_t leaf_level;      /* octree leaf level (src/main.cpp:204-211 uses 10); <= node_levels-1,
	                             and node_levels+1-leaf_level <= 8 (at most 2^24 voxels per leaf) */
	uint32_t keep_history;    /* 0: a rewritten leaf reuses its block when it fits (DAGColorPool) */
	uint64_t max_nodes;       /* octree node capacity (8 words each), <= 2^30 */
	uint64_t max_leaf_words;  /* leaf word capacity, <= 2^30 */
} hd_color_config;
typedef struct hd_vbr_edit_desc {
	hd_edit_desc edit;        /* op: HD_OP_FILL coloured fill, HD_OP_PAINT recolour (geometry kept),
	                             HD_OP_DIG stateless dig (colours kept, like the application's digs) */
	uint32_t colors;          /* VBRColor: RGB8 (r | g << 8 | b << 16) when bits_per_weight is 0, else
	                             two R5G6B5 end points (low 16 bits first) */
	uint32_t weight;          /* < 2^bits_per_weight (0 when bits_per_weight is 0) */
	uint32_t bits_per_weight; /* 0..3 */
	uint32_t pad;
} hd_vbr_edit_desc;           /* 56 bytes */
typedef struct hd_vbr_color {
	uint32_t has_value, colors, weight, bits_per_weight; /* VBRColor fields */
	float rgb[3];                                        /* trace.frag's colour (VBRColor::Get) */
} hd_vbr_color;               /* 28 bytes */
typedef struct hd_color_pool hd_color_pool;
/* A colour octree for the voxels of `pool` (device memory of pool's GPU).
 * Destroy it before `pool` if it is still to be edited; hd_color_pool_destroy,
 * hd_color_pool_read and hd_color_fetch do not touch the node pool. */
hd_status hd_color_pool_create(hd_pool *pool, const hd_color_config *cfg, hd_color_pool **out);
void hd_color_pool_destroy(hd_color_pool *cpool);
/* Host mirror: node count and leaf word count; with non-null buffers also the
 * nodes (8 words each) and the leaf words. */
hd_status hd_color_pool_read(hd_color_pool *cpool, uint32_t *nodes, uint64_t *n_nodes, uint32_t *leaves,
                             uint64_t *n_leaf_words);
/* Colour edits applied one after another (each the reference's Edit with a
 * VBREditorWrapper, or a stateless dig): the colour octree from the DAG as it
 * was before the edit, then the geometry through hd_edit.  Returns the new
 * DAG root and colour root.  HD_ERR_POOL_OOM when the octree is full: that
 * edit is not applied (both roots stay as after the previous edit). */
hd_status hd_vbr_edit(hd_pool *pool, hd_color_pool *cpool, uint32_t root, uint32_t color_root, const hd_vbr_edit_desc *edits,
                      uint32_t n, uint32_t *out_root, uint32_t *out_color_root);
/* Colours of n voxels (device buffers: xyz triples at voxel resolution) under
 * color_root (Color_Fetch, trace.frag:339-356).  Not ordered against a
 * concurrent hd_vbr_edit of the same colour pool. */
hd_status hd_color_fetch(hd_color_pool *cpool, uint32_t color_root, const uint32_t *d_xyz, uint32_t n,
                         hd_vbr_color *d_out, void *stream);


const char *hd_status_string(hd_status s);
/* 1 if a CUDA device is usable, else 0. */
int hd_device_available(void);

#ifdef __cplusplus
}
#endif

#endif /* HASHDAG_GPU_H */
