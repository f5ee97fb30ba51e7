// hd_engine.cu -- host side of the GB300 HashDAG edit engine: pool lifecycle,
// edit workspace, the launch sequence of one batched edit pass, find-or-insert
// of caller nodes, the host mirror (download / upload + index rebuild), point
// queries and the C ABI of include/hashdag_gpu.h.
#include "hd_internal.h"
#include "hd_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unordered_map>

using namespace hd;

hd_status hd_check(cudaError_t e) { return e == cudaSuccess ? HD_OK : HD_ERR_CUDA; }

#define HD_TRY(x)                                                                                                     \
	do {                                                                                                              \
		cudaError_t e_ = (x);                                                                                         \
		if (e_ != cudaSuccess) {                                                                                      \
			fprintf(stderr, "hashdag_gb300: %s failed: %s (%s:%d)\n", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
			return HD_ERR_CUDA;                                                                                       \
		}                                                                                                             \
	} while (0)

namespace {

// ------------------------------------------------------------------ config
uint64_t total_buckets_of(const hd_config &c) {
	uint64_t t = 0;
	for (uint32_t l = 0; l < c.node_levels; ++l)
		t += 1ull << c.bucket_bits_each_level[l];
	return t;
}

bool validate(const hd_config *c) {
	if (!c || c->node_levels < 1 || c->node_levels > kMaxNodeLevels)
		return false;
	if (c->word_bits_per_page < 4 || c->word_bits_per_page > 24) // Config::kMinWordBitsPerPage
		return false;
	if (c->hasher != HD_HASHER_MURMUR32 && c->hasher != HD_HASHER_ZERO)
		return false;
	for (uint32_t l = 0; l < c->node_levels; ++l)
		if (c->bucket_bits_each_level[l] > 31)
			return false;
	// Config::Validate (include/hashdag/Config.hpp:48-56): total words - 1 <= Word(-2)
	uint64_t tb = total_buckets_of(*c);
	uint32_t wbb = c->word_bits_per_page + c->page_bits_per_bucket;
	if (wbb >= 63 || tb > (1ull << (63 - wbb)))
		return false;
	uint64_t total_words = tb << wbb;
	return total_words - 1 <= 0xFFFFFFFEull;
}

// ------------------------------------------------------------------ workspace
template <typename T> hd_status ws_alloc(hd_ws_host &ws, T **p, uint64_t count) {
	void *q = nullptr;
	if (count == 0)
		count = 1;
	cudaError_t e = cudaMalloc(&q, count * sizeof(T));
	if (e != cudaSuccess) {
		fprintf(stderr, "hashdag_gb300: workspace cudaMalloc of %llu bytes failed: %s\n",
		        (unsigned long long)(count * sizeof(T)), cudaGetErrorString(e));
		return HD_ERR_CUDA;
	}
	ws.allocs.push_back(q);
	*p = static_cast<T *>(q);
	return HD_OK;
}

void ws_free_all(hd_ws_host &ws) {
	for (void *p : ws.allocs)
		cudaFree(p);
	ws.allocs.clear();
	ws.edits = nullptr;
	ws.edit_cap = 0;
	Workspace z{};
	ws.d = z;
}

hd_status alloc_items(hd_ws_host &ws, Items &it, uint64_t cap) {
	it.cap = cap;
	hd_status s;
	if ((s = ws_alloc(ws, &it.pos, cap)) || (s = ws_alloc(ws, &it.base, cap)) || (s = ws_alloc(ws, &it.parent, cap)) ||
	    (s = ws_alloc(ws, &it.lst_off, cap)) || (s = ws_alloc(ws, &it.lst_len, cap)) || (s = ws_alloc(ws, &it.res, cap)))
		return s;
	return HD_OK;
}

// Leaf candidates carry parent slot and result (bits in leaf_new).
hd_status alloc_leaf_candidates(hd_ws_host &ws, Items &it, uint64_t cap) {
	it = Items{};
	it.cap = cap;
	hd_status s;
	if ((s = ws_alloc(ws, &it.parent, cap)) || (s = ws_alloc(ws, &it.res, cap)))
		return s;
	return HD_OK;
}

// (Re)allocates the workspace with at least the given capacities; keeps the
// counters.  Frees the old one first.
// Slots of the leaf-pattern cache of the multi-kernel pass (16 MB: an 8-byte
// key and the pointer in 16 bytes per slot, small enough to stay in L2).
constexpr uint32_t kLeafCacheSlots = 1u << 20;

hd_status ws_reserve(hd_pool *pool, uint64_t inner_cap, uint64_t leaf_cap, uint64_t list_cap, uint32_t edit_cap) {
	hd_ws_host &ws = pool->ws;
	const Workspace &cur = ws.d;
	if (cur.ctr && cur.inner.cap >= inner_cap && cur.leaf.cap >= leaf_cap && cur.list_cap >= list_cap &&
	    ws.edit_cap >= edit_cap)
		return HD_OK;
	// child slots are u32 (inner index * 8 + child), list offsets are u32
	inner_cap = std::min<uint64_t>(std::max<uint64_t>(inner_cap, cur.inner.cap), (1ull << 29) - 1);
	leaf_cap = std::min<uint64_t>(std::max<uint64_t>(leaf_cap, cur.leaf.cap), (1ull << 31) - 1);
	list_cap = std::min<uint64_t>(std::max<uint64_t>(list_cap, cur.list_cap), 0xFFFFFFF0ull);
	edit_cap = std::max<uint32_t>(edit_cap, ws.edit_cap);
	cudaDeviceSynchronize();
	ws_free_all(ws);
	++pool->shape_gen; // a captured pass graph holds the old workspace pointers
	Workspace d{};
	hd_status s;
	if ((s = alloc_items(ws, d.inner, inner_cap)) || (s = alloc_leaf_candidates(ws, d.leaf, leaf_cap)) ||
	    (s = ws_alloc(ws, &d.bchild, inner_cap * 8)) || (s = ws_alloc(ws, &d.cnew, inner_cap * 8)) ||
	    (s = ws_alloc(ws, &d.leaf_new, leaf_cap)) || (s = ws_alloc(ws, &d.lists, list_cap)) ||
	    (s = ws_alloc(ws, &d.long_q, inner_cap)) || (s = ws_alloc(ws, &d.todo, inner_cap)) ||
	    (s = ws_alloc(ws, &d.todo_parent, inner_cap)) || (s = ws_alloc(ws, &d.leaf_cls, inner_cap)) ||
	    (s = ws_alloc(ws, &d.lc_key, 2ull * kLeafCacheSlots)) ||
	    (s = ws_alloc(ws, &d.ctr, (uint64_t)kWsCtrCount)) ||
	    (s = ws_alloc(ws, &ws.edits, (uint64_t)edit_cap))) {
		ws_free_all(ws);
		return s;
	}
	d.list_cap = list_cap;
	d.lc_mask = kLeafCacheSlots - 1u;
	d.long_threshold = 16;
	ws.edit_cap = edit_cap;
	ws.d = d;
	// cudaMemset runs on the legacy stream, which does not order against
	// non-blocking streams: wait for it, or a pass already queued on another
	// stream could see its counters zeroed half-way through
	HD_TRY(cudaMemset(d.ctr, 0, kWsCtrCount * sizeof(unsigned long long)));
	return hd_check(cudaDeviceSynchronize());
}

uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

uint32_t isqrt64(uint64_t v) {
	uint64_t r = (uint64_t)std::sqrt((double)v);
	while (r * r > v)
		--r;
	while ((r + 1) * (r + 1) <= v)
		++r;
	return (uint32_t)r;
}

// Voxel bounding box [lo, hi) of an edit, clipped to the grid.
bool edit_bbox(const hd_edit_desc &e, uint32_t res, uint32_t lo[3], uint32_t hi[3]) {
	for (int a = 0; a < 3; ++a) {
		int64_t l, h;
		if (e.shape == HD_SHAPE_AABB) {
			l = e.p0[a];
			h = e.p1[a];
		} else {
			int64_t r = isqrt64(e.r2);
			l = (int64_t)e.p0[a] - r;
			h = (int64_t)e.p0[a] + r + 1;
		}
		l = std::max<int64_t>(l, 0);
		h = std::min<int64_t>(h, res);
		if (h <= l)
			return false;
		lo[a] = (uint32_t)l;
		hi[a] = (uint32_t)h;
	}
	return true;
}

} // namespace

// Grid size per level of one pass: nodes of each level that intersect some
// edit's bounding box bound the frontier; a pass over a small edit launches
// small grids.
void hd_grid_for_levels(const hd_pool *pool, const hd_edit_desc *edits, uint32_t n, uint32_t *grid) {
	const uint32_t L = pool->cfg.node_levels, VL = L + 1, res = 1u << VL;
	const uint32_t max_grid = (uint32_t)pool->num_sms * 64u; // the launch sites cap per kernel family
	std::vector<double> bound(L, 0.0);
	if (!edits) {
		for (uint32_t l = 0; l < L; ++l)
			grid[l] = max_grid;
		return;
	}
	for (uint32_t i = 0; i < n; ++i) {
		uint32_t lo[3], hi[3];
		if (!edit_bbox(edits[i], res, lo, hi))
			continue;
		for (uint32_t l = 0; l < L; ++l) {
			uint32_t sh = VL - l;
			double c = 1.0;
			for (int a = 0; a < 3; ++a)
				c *= double(((hi[a] - 1) >> sh) - (lo[a] >> sh) + 1);
			bound[l] += c;
		}
	}
	for (uint32_t l = 0; l < L; ++l) {
		double b = std::min(bound[l], std::ldexp(1.0, (int)std::min<uint32_t>(3 * l, 60)));
		double g = std::ceil(b / kBlock);
		grid[l] = (uint32_t)std::max(1.0, std::min<double>(g, max_grid));
	}
}

namespace {

// hd_edit passes of at least this many edits replay the captured pass graph.
constexpr uint32_t kGraphMinEdits = 4096;

// Word offset of the pass descriptor (edit count, input root) in the pool's
// 16-word device scratch (d_out_root) and its pinned host mirror (h_small).
constexpr uint32_t kPassDescWord = 4;

// One-CTA passes: at most this many blocks' worth of level-(L-2) nodes
// (2048) and of nodes at any level (8192) by the bounding-box estimate.
constexpr uint32_t kSmallPassLeafGrid = 8, kSmallPassGrid = 32;

// Whether a pass with these host edits runs as one CTA (bounding-box grids).
bool small_pass_grids(const hd_pool *pool, const hd_edit_desc *host_edits, uint32_t n, const uint32_t *grid) {
	const uint32_t L = pool->cfg.node_levels;
	if (!host_edits || n > std::max(1u, pool->tune.long_threshold) || L < 2)
		return false;
	bool small = grid[L - 2] <= kSmallPassLeafGrid;
	for (uint32_t l = 0; l < L; ++l)
		small = small && grid[l] <= kSmallPassGrid;
	return small;
}

// Launch sequence of one pass.  edits = device array of n edits; root from
// root_ptr (device) when non-null, else root_val.  host_edits (optional) sizes
// the grids.
// capture: enqueue for a CUDA graph (edit count and root from the pass
// descriptor, grids at their caps, long-list kernels always present, no waits,
// events or records).
hd_status launch_pass(hd_pool *pool, const hd_edit_desc *d_edits, uint32_t n, uint32_t root_val,
                      const uint32_t *root_ptr, uint32_t *d_out, cudaStream_t st, const hd_edit_desc *host_edits,
                      bool capture = false) {
	const uint32_t L = pool->cfg.node_levels;
	Workspace W = pool->ws.d;
	W.edits = d_edits;
	W.n_edits = n;
	W.long_threshold = std::max(1u, pool->tune.long_threshold);
	if (capture) {
		W.pass_desc = pool->d_out_root + kPassDescWord;
		root_ptr = W.pass_desc + 1;
		host_edits = nullptr;
	}
	const DevPool &P = pool->P;
	uint32_t grid[HD_MAX_LEVELS];
	hd_grid_for_levels(pool, host_edits, n, grid);
	const uint32_t sms = (uint32_t)pool->num_sms;
	const uint32_t long_grid = sms * std::max(1u, pool->tune.long_blocks_per_sm);
	const auto cap = [&](uint32_t g, uint32_t per_sm) { return std::max(1u, std::min(g, sms * std::max(1u, per_sm))); };
	// a pass that is small (grids sized from the edits' bounding boxes) and has
	// no long lists runs as one CTA: one launch instead of 3L+1
	if (!capture && pool->prof_passes >= pool->prof_max_passes && small_pass_grids(pool, host_edits, n, grid)) {
		{
			HD_TRY(cudaStreamWaitEvent(st, pool->ws_free, 0));
			HD_TRY(cudaMemsetAsync(W.ctr, 0, kWsCtrCount * sizeof(unsigned long long), st));
			W.lc_key = nullptr; // a one-CTA pass has too few leaves to pay for clearing the cache
			k_small_pass<<<1, kBlock, 0, st>>>(P, W, root_val, root_ptr, d_out);
			pool->kernel_launches += 1;
			HD_TRY(cudaGetLastError());
			HD_TRY(cudaEventRecord(pool->ws_free, st));
			return HD_OK;
		}
	}
	static const bool debug_env = getenv("HD_DEBUG_SYNC") != nullptr;
	const bool debug_sync = debug_env && !capture;
	cudaEvent_t *ev = nullptr;
	if (!capture && pool->prof_passes < pool->prof_max_passes)
		ev = pool->prof_events.data() + (uint64_t)pool->prof_passes++ * hd_prof_events_per_pass(L);
	uint32_t e = 0;
	auto mark = [&]() {
		if (ev)
			cudaEventRecord(ev[e++], st);
	};
	auto dbg = [&](const char *what, uint32_t l) {
		if (!debug_sync)
			return;
		cudaError_t err = cudaStreamSynchronize(st);
		unsigned long long c[kWsCtrCount];
		cudaMemcpy(c, W.ctr, sizeof(c), cudaMemcpyDeviceToHost);
		uint32_t perr = 0;
		cudaMemcpy(&perr, pool->P.counters + kCtrError, 4, cudaMemcpyDeviceToHost);
		fprintf(stderr,
		        "hd_debug %s l=%u err=%s ws_err=%llu pool_err=%u items=%llu list=%llu long=%llu max_probe=%llu "
		        "probe_steps=%llu cas_retry=%llu\n",
		        what, l, cudaGetErrorString(err), c[kWsError], perr, l < HD_MAX_LEVELS ? c[kWsItems + l] : 0ull,
		        c[kWsList], l < HD_MAX_LEVELS ? c[kWsLong + l] : 0ull, c[kWsMaxProbe], c[kWsProbeSteps], c[kWsCasRetry]);
	};
	if (!capture)
		HD_TRY(cudaStreamWaitEvent(st, pool->ws_free, 0));
	mark();
	HD_TRY(cudaMemsetAsync(W.ctr, 0, kWsCtrCount * sizeof(unsigned long long), st));
	if (W.lc_key) { // the leaf-pattern cache names leaves of this pool state only
		HD_TRY(cudaMemsetAsync(W.lc_key, 0, 2ull * (W.lc_mask + 1ull) * sizeof(unsigned long long), st));
	}
	k_root<<<1, kLongBlock, 0, st>>>(P, W, root_val, root_ptr);
	dbg("root", 0);
	uint64_t launches = 1;
	const bool longs = capture || n > W.long_threshold; // no list can be longer than the batch
	for (uint32_t l = 0; l + 2 < L; ++l) {
		k_expand_short<<<cap(grid[l], pool->tune.expand_blocks_per_sm), kBlock, 0, st>>>(P, W, l);
		dbg("expand_short", l + 1);
		++launches;
		if (longs) {
			k_expand_long<<<long_grid, kLongBlock, 0, st>>>(P, W, l);
			dbg("expand_long", l + 1);
			++launches;
		}
	}
	mark();
	if (L >= 2) {
		if (pool->tune.leaf_compact)
			k_leafparent_compact<<<cap(grid[L - 2], pool->tune.leaf_blocks_per_sm), kBlock, 0, st>>>(P, W);
		else
			k_leafparent_short<<<cap(grid[L - 2], pool->tune.leaf_blocks_per_sm), kBlock, 0, st>>>(P, W);
		dbg("leafparent_short", L - 1);
		++launches;
		if (longs) {
			k_leafparent_long<<<long_grid, kBlock, 0, st>>>(P, W);
			dbg("leafparent_long", L - 1);
			++launches;
		}
	}
	mark();
	const uint32_t dq = pool->tune.dedup_blocks_per_sm;
	k_dedup<true><<<cap(grid[L - 1], dq), kBlock, 0, st>>>(P, W, L - 1, 0u);
	dbg("dedup_leaf", L - 1);
	mark();
	for (uint32_t l = L - 1; l-- > 0;) {
		const uint32_t todo = l + 2 == L ? 1u : 0u; // level L-2 runs over the unresolved nodes only
		k_dedup<false><<<cap(grid[l], dq), kBlock, 0, st>>>(P, W, l, todo);
		dbg("dedup", l);
		mark();
	}
	k_finish<<<1, 32, 0, st>>>(P, W, d_out);
	mark();
	launches += 1 + (uint64_t)L;
	HD_TRY(cudaGetLastError());
	if (capture) {
		pool->pass_graph_kernels = (uint32_t)launches;
		return HD_OK;
	}
	pool->kernel_launches += launches;
	HD_TRY(cudaEventRecord(pool->ws_free, st));
	return HD_OK;
}

// The multi-kernel pass of hd_edit as a CUDA graph: captured once per
// workspace allocation and launch shape on a private stream, replayed with the
// edit count and root written into the pinned pass descriptor first.  Nodes:
// descriptor upload, error-word clear, the pass's kernels, counter and error
// downloads into the pinned buffers run_pass_sync reads.
hd_status pass_graph(hd_pool *pool, cudaGraphExec_t *out) {
	if (pool->pass_graph && pool->graph_gen == pool->shape_gen) {
		*out = pool->pass_graph;
		return HD_OK;
	}
	if (pool->pass_graph) {
		cudaGraphExecDestroy(pool->pass_graph);
		pool->pass_graph = nullptr;
	}
	if (!pool->capture_stream)
		HD_TRY(cudaStreamCreateWithFlags(&pool->capture_stream, cudaStreamNonBlocking));
	// With lazy module loading a kernel is loaded at its first launch, which a
	// capturing stream does not allow (a serving scene can capture before the
	// process ever launched the long-list kernels): load every kernel first.
	cudaFuncAttributes fa;
	HD_TRY(cudaFuncGetAttributes(&fa, k_root));
	HD_TRY(cudaFuncGetAttributes(&fa, k_expand_short));
	HD_TRY(cudaFuncGetAttributes(&fa, k_expand_long));
	HD_TRY(cudaFuncGetAttributes(&fa, k_leafparent_short));
	HD_TRY(cudaFuncGetAttributes(&fa, k_leafparent_compact));
	HD_TRY(cudaFuncGetAttributes(&fa, k_leafparent_long));
	HD_TRY(cudaFuncGetAttributes(&fa, k_dedup<true>));
	HD_TRY(cudaFuncGetAttributes(&fa, k_dedup<false>));
	HD_TRY(cudaFuncGetAttributes(&fa, k_finish));
	cudaStream_t cs = pool->capture_stream;
	HD_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
	hd_status s = HD_OK;
	if (cudaMemcpyAsync(pool->d_out_root + kPassDescWord, pool->h_small + kPassDescWord, 8, cudaMemcpyHostToDevice,
	                    cs) != cudaSuccess ||
	    cudaMemsetAsync(pool->P.counters + kCtrError, 0, 4, cs) != cudaSuccess)
		s = HD_ERR_CUDA;
	if (!s)
		s = launch_pass(pool, pool->ws.edits, 0, kNull, nullptr, pool->d_out_root, cs, nullptr, true);
	if (!s && (cudaMemcpyAsync(pool->ws.ctr_host, pool->ws.d.ctr, kWsCtrCount * sizeof(unsigned long long),
	                           cudaMemcpyDeviceToHost, cs) != cudaSuccess ||
	           cudaMemcpyAsync(pool->h_small, pool->P.counters + kCtrError, 4, cudaMemcpyDeviceToHost, cs) !=
	               cudaSuccess))
		s = HD_ERR_CUDA;
	cudaGraph_t g = nullptr;
	const cudaError_t ec = cudaStreamEndCapture(cs, &g);
	if (!s && ec != cudaSuccess)
		s = HD_ERR_CUDA;
	cudaGraphExec_t exec = nullptr;
	if (!s && cudaGraphInstantiate(&exec, g, 0) != cudaSuccess)
		s = HD_ERR_CUDA;
	if (g)
		cudaGraphDestroy(g);
	if (s) {
		cudaGetLastError();
		return s;
	}
	pool->pass_graph = exec;
	pool->graph_gen = pool->shape_gen;
	*out = exec;
	return HD_OK;
}

__global__ void k_error_from_ws(DevPool P, Workspace W) {
	if (threadIdx.x == 0 && W.ctr[kWsError])
		set_error(&P.counters[kCtrError], (u32)W.ctr[kWsError]);
}

hd_status status_of(uint32_t err) {
	switch (err) {
	case 0:
		return HD_OK;
	case kErrBucketFull:
		return HD_ERR_BUCKET_FULL;
	case kErrOom:
		return HD_ERR_POOL_OOM;
	case kErrIndexFull:
		return HD_ERR_INDEX_FULL;
	case kErrCapacity:
		return HD_ERR_CAPACITY;
	case kErrTimeout:
		return HD_ERR_TIMEOUT;
	case kErrInternal:
		return HD_ERR_INTERNAL;
	case kErrInvalidRoot:
		return HD_ERR_INVALID_ARG;
	default:
		return HD_ERR_CUDA;
	}
}

// Synchronous pass with workspace growth on overflow.  Host edits are copied
// into the workspace on every attempt (growing the workspace reallocates it).
hd_status run_pass_sync(hd_pool *pool, const hd_edit_desc *h_edits, uint32_t n, uint32_t root, uint32_t *out_root,
                        cudaStream_t st) {
	const uint32_t L = pool->cfg.node_levels;
	static const bool debug_env = getenv("HD_DEBUG_SYNC") != nullptr;
	for (int attempt = 0; attempt < 24; ++attempt) {
		// large passes replay the captured multi-kernel graph (its grids are the
		// caps, which large passes reach anyway); smaller ones launch with grids
		// sized from the edits' bounding boxes, which a graph cannot follow
		cudaGraphExec_t graph = nullptr;
		if (n >= kGraphMinEdits && pool->prof_passes >= pool->prof_max_passes && !debug_env &&
		    pass_graph(pool, &graph) != HD_OK)
			graph = nullptr;
		HD_TRY(cudaStreamWaitEvent(st, pool->ws_free, 0));
		if (graph) {
			pool->h_small[kPassDescWord] = n;
			pool->h_small[kPassDescWord + 1] = root;
			HD_TRY(cudaMemcpyAsync(pool->ws.edits, h_edits, n * sizeof(hd_edit_desc), cudaMemcpyHostToDevice, st));
			HD_TRY(cudaGraphLaunch(graph, st));
			pool->kernel_launches += pool->pass_graph_kernels;
			HD_TRY(cudaEventRecord(pool->ws_free, st));
		} else {
			HD_TRY(cudaMemsetAsync(pool->P.counters + kCtrError, 0, 4, st));
			HD_TRY(cudaMemcpyAsync(pool->ws.edits, h_edits, n * sizeof(hd_edit_desc), cudaMemcpyHostToDevice, st));
			hd_status s = launch_pass(pool, pool->ws.edits, n, root, nullptr, pool->d_out_root, st, h_edits);
			if (s)
				return s;
			HD_TRY(cudaMemcpyAsync(pool->ws.ctr_host, pool->ws.d.ctr, kWsCtrCount * sizeof(unsigned long long),
			                       cudaMemcpyDeviceToHost, st));
			HD_TRY(cudaMemcpyAsync(pool->h_small, pool->P.counters + kCtrError, 4, cudaMemcpyDeviceToHost, st));
		}
		HD_TRY(cudaStreamSynchronize(st));
		const unsigned long long *c = pool->ws.ctr_host;
		for (uint32_t l = 0; l < L; ++l) {
			pool->last_items[l] = c[kWsItems + l];
			pool->last_cand[l] = c[kWsCand + l];
			pool->last_ins[l] = c[kWsIns + l];
		}
		if (c[kWsError] == kErrInvalidRoot || c[kWsError] == kErrInternal) {
			*out_root = root;
			return status_of((uint32_t)c[kWsError]);
		}
		if (c[kWsError] == kErrCapacity) {
			uint64_t inner = 0;
			for (uint32_t l = 0; l + 1 < L; ++l)
				inner += c[kWsItems + l];
			uint64_t leaf = c[kWsItems + L - 1], list = c[kWsList];
			const Workspace &d = pool->ws.d;
			uint64_t ni = inner > d.inner.cap ? std::max<uint64_t>(inner * 2, d.inner.cap * 2) : d.inner.cap;
			uint64_t nl = leaf > d.leaf.cap ? std::max<uint64_t>(leaf * 2, d.leaf.cap * 2) : d.leaf.cap;
			uint64_t nli = list > d.list_cap ? std::max<uint64_t>(list * 2, d.list_cap * 2) : d.list_cap;
			if (ni == d.inner.cap && nl == d.leaf.cap && nli == d.list_cap)
				ni *= 2; // should not happen; grow something
			hd_status g = ws_reserve(pool, ni, nl, nli, pool->ws.edit_cap);
			if (g)
				return g;
			continue;
		}
		*out_root = (uint32_t)c[kWsRoot];
		uint32_t err = pool->h_small[0];
		if (err) {
			*out_root = root;
			return status_of(err);
		}
		return HD_OK;
	}
	*out_root = root;
	return HD_ERR_CAPACITY;
}

// ------------------------------------------------------------------ index rebuild
// Walks every bucket like NodePool.hpp:79-132 (find_node over all words) and
// inserts each node into the dedup index.
__global__ void k_index_rebuild(DevPool P, u32 total_buckets) {
	const u32 L = P.cfg.L, wp = wpp(P.cfg);
	const u64 stride = (u64)gridDim.x * blockDim.x;
	for (u64 b = (u64)blockIdx.x * blockDim.x + threadIdx.x; b < total_buckets; b += stride) {
		u32 level = 0;
		for (u32 l = 0; l < L; ++l)
			if (b >= P.cfg.bucket_base[l])
				level = l;
		const bool leaf = level == L - 1;
		const u32 bw = P.bucket_words[b];
		u32 off = 0;
		while (off < bw) {
			const u32 ptr = ((u32)b << (P.cfg.wbpp + P.cfg.pbpb)) | off;
			const u32 phys = P.page_table[ptr >> P.cfg.wbpp];
			if (phys == kUnallocPage || page_lost(P, phys)) { // page lost: skip it
				off = (off | (wp - 1u)) + 1u;
				continue;
			}
			const u32 *p = P.heap + ((u64)phys << P.cfg.wbpp) + (off & (wp - 1u));
			u32 n;
			u32 h;
			if (leaf) {
				n = 2;
				h = hash_leaf((u64)p[0] | ((u64)p[1] << 32));
			} else {
				const u32 m = p[0] & 0xFFu;
				if (!m) { // zero padding: the rest of the page is empty
					off = (off | (wp - 1u)) + 1u;
					continue;
				}
				n = __popc(m) + 1u;
				Murmur mm;
				for (u32 k = 0; k < n; ++k)
					mm.add(p[k]);
				h = mm.finish(n);
			}
			if ((off & (wp - 1u)) + n > wp) { // malformed: node would straddle
				set_error(&P.counters[kCtrError], kErrIndexFull);
				break;
			}
			const unsigned long long tag = (unsigned long long)(h & 0x7FFFFFFFu) << 32;
			u64 s = index_start(h, level, P.index_mask);
			for (u64 probe = 0; probe <= P.index_mask; ++probe, s = (s + 1) & P.index_mask) {
				unsigned long long prev = atomicCAS(&P.index[s], kSlotEmpty, tag | ptr);
				if (prev == kSlotEmpty) {
					atomicAdd(&P.counters[kCtrIndexUsed], 1u);
					break;
				}
				if (((prev >> 32) & 0x7FFFFFFFull) == (tag >> 32) && !(prev >> 63)) {
					const u32 other = (u32)prev;
					if ((other >> (P.cfg.wbpp + P.cfg.pbpb)) == (u32)b) {
						const u32 *q = node_addr(P, other);
						bool eq = true;
						for (u32 k = 0; k < n; ++k)
							eq &= q[k] == p[k];
						if (eq)
							break; // duplicate content: keep the first
					}
				}
				if (probe == P.index_mask)
					set_error(&P.counters[kCtrError], kErrIndexFull);
			}
			off += n;
		}
	}
}

// ------------------------------------------------------------------ queries
__global__ void k_query(DevPool P, u32 root, const u32 *xyz, u32 n, uint8_t *out) {
	const u32 L = P.cfg.L, VL = L + 1;
	for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
		const u32 x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
		u32 ptr = root;
		bool v = ptr != kNull;
		for (u32 l = 0; v && l + 1 < L; ++l) {
			const u32 sh = VL - l - 1;
			const u32 c = ((x >> sh) & 1u) | (((y >> sh) & 1u) << 1) | (((z >> sh) & 1u) << 2);
			const u32 *p = node_addr(P, ptr);
			const u32 m = p[0] & 0xFFu;
			if (!((m >> c) & 1u)) {
				v = false;
				break;
			}
			ptr = p[1 + __popc(m & ((1u << c) - 1u))];
		}
		if (v) {
			const u32 *p = node_addr(P, ptr);
			const u32 b = (((x >> 1) & 1u) << 3) | (((y >> 1) & 1u) << 4) | (((z >> 1) & 1u) << 5) | (x & 1u) |
			              ((y & 1u) << 1) | ((z & 1u) << 2);
			v = (p[b >> 5] >> (b & 31u)) & 1u;
		}
		out[i] = v ? 1 : 0;
	}
}

// Gather virtual pages into a contiguous device buffer.
__global__ void k_gather_pages(DevPool P, const u32 *vpages, u32 n, u32 *dst) {
	const u32 wp = wpp(P.cfg);
	for (u64 w = (u64)blockIdx.x * blockDim.x + threadIdx.x; w < (u64)n * wp; w += (u64)gridDim.x * blockDim.x) {
		const u64 i = w / wp, k = w % wp;
		const u32 phys = P.page_table[vpages[i]];
		dst[w] = phys == kUnallocPage ? 0u : P.heap[((u64)phys << P.cfg.wbpp) + k];
	}
}

__global__ void k_max_reduce(const u32 *a, u64 n, u32 *out) {
	u32 m = 0;
	for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
		m = max(m, a[i]);
	m = __reduce_max_sync(0xFFFFFFFFu, m);
	if ((threadIdx.x & 31) == 0)
		atomicMax(out, m);
}

// Find-or-insert of host nodes at one level (no stream argument: synchronous).
hd_status upsert_impl(hd_pool *pool, uint32_t level, const uint32_t *words, const uint32_t *lens, uint32_t n,
                      uint32_t *out) {
	const uint32_t L = pool->cfg.node_levels;
	if (level >= L || (n && (!words || !lens || !out)))
		return HD_ERR_INVALID_ARG;
	if (n == 0)
		return HD_OK;
	const bool leaf = level == L - 1;
	std::vector<uint64_t> leafbits;
	std::vector<uint32_t> cnew, bchild;
	uint64_t o = 0;
	for (uint32_t i = 0; i < n; ++i) {
		const uint32_t len = lens[i];
		if (leaf) {
			if (len != 2)
				return HD_ERR_INVALID_ARG;
			leafbits.push_back((uint64_t)words[o] | ((uint64_t)words[o + 1] << 32));
		} else {
			const uint32_t m = words[o];
			if (m == 0 || m > 0xFFu || len != (uint32_t)__builtin_popcount(m) + 1u)
				return HD_ERR_INVALID_ARG;
			uint32_t k = 1;
			for (int c = 0; c < 8; ++c) {
				uint32_t v = kNull;
				if ((m >> c) & 1u) {
					v = words[o + k++];
					if (v == kNull)
						return HD_ERR_INVALID_ARG;
				}
				cnew.push_back(v);
				bchild.push_back(0xFFFFFFFEu); // never equal: always a candidate
			}
		}
		o += len;
	}
	hd_status s = ws_reserve(pool, leaf ? 1 : n, leaf ? n : 1, 1, 1);
	if (s)
		return s;
	Workspace W = pool->ws.d;
	Items &it = leaf ? W.leaf : W.inner;
	cudaStream_t st = 0;
	std::vector<uint32_t> parents(n, kNull);
	std::vector<unsigned long long> ctr(kWsCtrCount, 0ull);
	ctr[kWsItems + level] = n;
	HD_TRY(cudaStreamWaitEvent(st, pool->ws_free, 0));
	HD_TRY(cudaMemcpyAsync(W.ctr, ctr.data(), kWsCtrCount * 8, cudaMemcpyHostToDevice, st));
	HD_TRY(cudaMemcpyAsync(it.parent, parents.data(), n * 4ull, cudaMemcpyHostToDevice, st));
	if (leaf) {
		HD_TRY(cudaMemcpyAsync(W.leaf_new, leafbits.data(), n * 8ull, cudaMemcpyHostToDevice, st));
	} else {
		HD_TRY(cudaMemcpyAsync(W.cnew, cnew.data(), n * 32ull, cudaMemcpyHostToDevice, st));
		HD_TRY(cudaMemcpyAsync(W.bchild, bchild.data(), n * 32ull, cudaMemcpyHostToDevice, st));
	}
	const uint32_t grid = std::max(1u, std::min(ceil_div(n, kBlock), (uint32_t)pool->num_sms * 8u));
	if (leaf)
		k_dedup<true><<<grid, kBlock, 0, st>>>(pool->P, W, level, 0u);
	else
		k_dedup<false><<<grid, kBlock, 0, st>>>(pool->P, W, level, 0u);
	k_finish<<<1, 32, 0, st>>>(pool->P, W, nullptr);
	pool->kernel_launches += 2;
	HD_TRY(cudaGetLastError());
	HD_TRY(cudaEventRecord(pool->ws_free, st));
	HD_TRY(cudaMemcpyAsync(out, it.res, n * 4ull, cudaMemcpyDeviceToHost, st));
	HD_TRY(cudaMemcpyAsync(pool->h_small, pool->P.counters + kCtrError, 4, cudaMemcpyDeviceToHost, st));
	HD_TRY(cudaStreamSynchronize(st));
	return status_of(pool->h_small[0]);
}

hd_status make_filled(hd_pool *pool) {
	const uint32_t L = pool->cfg.node_levels;
	++pool->shape_gen; // the filled pointers are kernel parameters of a captured pass graph
	uint32_t leaf[2] = {kNull, kNull}, two = 2, nine = 9, r;
	hd_status s = upsert_impl(pool, L - 1, leaf, &two, 1, &r);
	if (s)
		return s;
	pool->P.cfg.filled[L - 1] = r;
	for (uint32_t l = L - 1; l-- > 0;) {
		uint32_t node[9] = {0xFFu, r, r, r, r, r, r, r, r};
		s = upsert_impl(pool, l, node, &nine, 1, &r);
		if (s)
			return s;
		pool->P.cfg.filled[l] = r;
	}
	return HD_OK;
}

void pool_free(hd_pool *p) {
	if (!p)
		return;
	cudaSetDevice(p->device);
	cudaDeviceSynchronize();
	ws_free_all(p->ws);
	cudaFree(p->P.bucket_words);
	cudaFree(p->P.page_table);
	cudaFree(p->P.heap);
	cudaFree(p->P.counters);
	cudaFree(p->P.index);
	cudaFree(p->d_out_root);
	if (p->h_small)
		cudaFreeHost(p->h_small);
	if (p->ws.ctr_host)
		cudaFreeHost(p->ws.ctr_host);
	if (p->ws_free)
		cudaEventDestroy(p->ws_free);
	if (p->pass_graph)
		cudaGraphExecDestroy(p->pass_graph);
	if (p->capture_stream)
		cudaStreamDestroy(p->capture_stream);
	for (cudaEvent_t e : p->prof_events)
		cudaEventDestroy(e);
	cudaFree(p->ck_bucket_words);
	cudaFree(p->ck_page_table);
	cudaFree(p->ck_counters);
	cudaFree(p->ck_index);
	delete p;
}

uint64_t sphere_count(int64_t cx, int64_t cy, int64_t cz, uint64_t r2, int64_t res) {
	const int64_t r = isqrt64(r2);
	uint64_t total = 0;
	for (int64_t x = std::max<int64_t>(0, cx - r); x <= std::min<int64_t>(res - 1, cx + r); ++x) {
		const uint64_t rx = r2 - (uint64_t)((x - cx) * (x - cx));
		const int64_t yr = isqrt64(rx);
		int64_t zr = yr;
		// walk |dy| upwards; the z half-width only shrinks
		for (int64_t dy = 0; dy <= yr; ++dy) {
			const uint64_t rem = rx - (uint64_t)(dy * dy);
			while ((uint64_t)(zr * zr) > rem)
				--zr;
			const int64_t z0 = std::max<int64_t>(0, cz - zr), z1 = std::min<int64_t>(res - 1, cz + zr);
			const uint64_t cnt = z1 >= z0 ? (uint64_t)(z1 - z0 + 1) : 0;
			for (int s = 0; s < (dy ? 2 : 1); ++s) {
				const int64_t y = s ? cy - dy : cy + dy;
				if (y >= 0 && y < res)
					total += cnt;
			}
		}
	}
	return total;
}

} // namespace

// Internal entry points shared with the other translation units (device
// current, pool lock held, no pass in flight).
hd_status hd_rebuild_index(hd_pool *pool, cudaStream_t st) {
	HD_TRY(cudaMemsetAsync(pool->P.index, 0xFF, (pool->P.index_mask + 1) * 8, st));
	HD_TRY(cudaMemsetAsync(pool->P.counters + kCtrError, 0, 8, st)); // error word and index usage
	k_index_rebuild<<<std::max(1u, std::min(ceil_div(pool->total_buckets, 256), 8192u)), 256, 0, st>>>(
	    pool->P, (uint32_t)pool->total_buckets);
	HD_TRY(cudaGetLastError());
	HD_TRY(cudaMemcpyAsync(pool->h_small, pool->P.counters + kCtrError, 4, cudaMemcpyDeviceToHost, st));
	HD_TRY(cudaStreamSynchronize(st));
	const uint32_t err = pool->h_small[0];
	return err ? status_of(err) : HD_OK;
}

hd_status hd_remake_filled(hd_pool *pool) { return make_filled(pool); }

// ====================================================================== C ABI
extern "C" {

int hd_config_validate(const hd_config *config) { return validate(config) ? 1 : 0; }

void hd_config_default(uint32_t level_count, uint32_t top_level_count, uint32_t word_bits_per_page,
                       uint32_t page_bits_per_bucket, uint32_t bucket_bits_per_top_level,
                       uint32_t bucket_bits_per_bottom_level, hd_config *out) {
	// DefaultConfig<Word>::operator() (include/hashdag/Config.hpp:59-75)
	std::memset(out, 0, sizeof(*out));
	out->word_bits_per_page = word_bits_per_page;
	out->page_bits_per_bucket = page_bits_per_bucket;
	out->hasher = HD_HASHER_MURMUR32;
	uint32_t n = 0;
	for (uint32_t l = 0; l + 1 < level_count && n < HD_MAX_LEVELS; ++l)
		out->bucket_bits_each_level[n++] = l < top_level_count ? bucket_bits_per_top_level : bucket_bits_per_bottom_level;
	out->node_levels = n;
}

int hd_device_available(void) {
	int n = 0;
	return cudaGetDeviceCount(&n) == cudaSuccess && n > 0 ? 1 : 0;
}

const char *hd_status_string(hd_status s) {
	switch (s) {
	case HD_OK:
		return "ok";
	case HD_ERR_INVALID_ARG:
		return "invalid argument";
	case HD_ERR_BUCKET_FULL:
		return "bucket full";
	case HD_ERR_POOL_OOM:
		return "device page heap exhausted";
	case HD_ERR_INDEX_FULL:
		return "dedup index full";
	case HD_ERR_CAPACITY:
		return "edit workspace capacity exceeded";
	case HD_ERR_CUDA:
		return "CUDA error";
	case HD_ERR_TIMEOUT:
		return "device wait timed out";
	case HD_ERR_NO_DEVICE:
		return "no CUDA device";
	case HD_ERR_INTERNAL:
		return "device consistency check failed";
	}
	return "unknown";
}

hd_status hd_pool_create(const hd_config *config, uint64_t heap_pages, uint32_t index_log2, int device,
                         hd_pool **out_pool) {
	if (!out_pool)
		return HD_ERR_INVALID_ARG;
	*out_pool = nullptr;
	if (!validate(config) || heap_pages < 2 || heap_pages > 0xFFFFFFF0ull)
		return HD_ERR_INVALID_ARG;
	if (!hd_device_available())
		return HD_ERR_NO_DEVICE;
	HD_TRY(cudaSetDevice(device));
	hd_pool *p = new hd_pool();
	p->device = device;
	p->cfg = *config;
	cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, device);
	DevConfig &c = p->P.cfg;
	c.wbpp = config->word_bits_per_page;
	c.pbpb = config->page_bits_per_bucket;
	c.L = config->node_levels;
	c.hasher = config->hasher;
	uint32_t base = 0;
	for (uint32_t l = 0; l < c.L; ++l) {
		c.bucket_bits[l] = config->bucket_bits_each_level[l];
		c.bucket_base[l] = base;
		base += 1u << c.bucket_bits[l];
		c.filled[l] = kNull;
	}
	p->total_buckets = total_buckets_of(*config);
	p->total_pages = p->total_buckets << c.pbpb;
	p->P.total_pages = p->total_pages;
	// a heap that can hold every virtual page is identity-mapped: node reads skip the page table
	if (heap_pages >= p->total_pages) {
		heap_pages = p->total_pages;
		p->P.identity = 1;
	}
	const uint64_t heap_words = heap_pages << c.wbpp;
	uint64_t slots = 1;
	if (index_log2)
		slots = 1ull << std::min<uint32_t>(index_log2, 31); // slot numbers are carried as u32
	else
		while (slots < std::max<uint64_t>(heap_words / 2, 1024))
			slots <<= 1;
	p->P.heap_pages = (uint32_t)heap_pages;
	p->P.index_mask = slots - 1;
	auto fail = [&](hd_status s) {
		pool_free(p);
		return s;
	};
	if (cudaMalloc(&p->P.bucket_words, p->total_buckets * 4) != cudaSuccess ||
	    cudaMalloc(&p->P.page_table, p->total_pages * 4) != cudaSuccess ||
	    cudaMalloc(&p->P.heap, heap_words * 4) != cudaSuccess ||
	    cudaMalloc(&p->P.counters, kCtrCount * 4) != cudaSuccess ||
	    cudaMalloc(&p->P.index, slots * 8) != cudaSuccess || cudaMalloc(&p->d_out_root, 64) != cudaSuccess ||
	    cudaMallocHost(&p->h_small, 64) != cudaSuccess ||
	    cudaMallocHost(&p->ws.ctr_host, kWsCtrCount * sizeof(unsigned long long)) != cudaSuccess ||
	    cudaEventCreateWithFlags(&p->ws_free, cudaEventDisableTiming) != cudaSuccess) {
		cudaGetLastError();
		return fail(HD_ERR_POOL_OOM);
	}
	uint32_t ctr0[kCtrCount] = {1u, 0u, 0u, 0u}; // physical page 0 stays the zero page
	if (cudaMemset(p->P.bucket_words, 0, p->total_buckets * 4) != cudaSuccess ||
	    cudaMemset(p->P.page_table, 0xFF, p->total_pages * 4) != cudaSuccess ||
	    cudaMemset(p->P.heap, 0, heap_words * 4) != cudaSuccess ||
	    cudaMemset(p->P.index, 0xFF, slots * 8) != cudaSuccess ||
	    cudaMemcpy(p->P.counters, ctr0, sizeof(ctr0), cudaMemcpyHostToDevice) != cudaSuccess)
		return fail(HD_ERR_CUDA);
	hd_status s = ws_reserve(p, 1u << 14, 1u << 16, 1u << 18, 64);
	if (s)
		return fail(s);
	s = make_filled(p);
	if (s)
		return fail(s);
	*out_pool = p;
	return HD_OK;
}

void hd_pool_destroy(hd_pool *pool) { pool_free(pool); }

hd_status hd_pool_filled_pointers(const hd_pool *pool, uint32_t *out) {
	if (!pool || !out)
		return HD_ERR_INVALID_ARG;
	for (uint32_t l = 0; l < pool->cfg.node_levels; ++l)
		out[l] = pool->P.cfg.filled[l];
	return HD_OK;
}

hd_status hd_pool_get_error(const hd_pool *pool, uint32_t *out_error) {
	if (!pool || !out_error)
		return HD_ERR_INVALID_ARG;
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	HD_TRY(cudaMemcpy(out_error, pool->P.counters + kCtrError, 4, cudaMemcpyDeviceToHost));
	return HD_OK;
}

hd_status hd_pool_clear_error(hd_pool *pool) {
	if (!pool)
		return HD_ERR_INVALID_ARG;
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	HD_TRY(cudaMemset(pool->P.counters + kCtrError, 0, 4));
	return hd_check(cudaDeviceSynchronize());
}

hd_status hd_pool_get_stats(const hd_pool *pool, hd_pool_stats *out) {
	if (!pool || !out)
		return HD_ERR_INVALID_ARG;
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	uint32_t ctr[kCtrCount];
	HD_TRY(cudaMemcpy(ctr, pool->P.counters, sizeof(ctr), cudaMemcpyDeviceToHost));
	uint32_t *d_max = nullptr, mx = 0;
	HD_TRY(cudaMalloc(&d_max, 4));
	cudaMemset(d_max, 0, 4);
	k_max_reduce<<<256, 256>>>(pool->P.bucket_words, pool->total_buckets, d_max);
	cudaError_t e = cudaMemcpy(&mx, d_max, 4, cudaMemcpyDeviceToHost);
	cudaFree(d_max);
	HD_TRY(e);
	out->heap_pages = pool->P.heap_pages;
	out->used_pages = std::min<uint64_t>(ctr[kCtrHeapNext], pool->P.heap_pages) - 1;
	out->total_buckets = pool->total_buckets;
	out->total_pages = pool->total_pages;
	out->index_slots = pool->P.index_mask + 1;
	out->index_used = ctr[kCtrIndexUsed];
	out->max_bucket_words = mx;
	out->words_per_bucket = 1u << (pool->P.cfg.wbpp + pool->P.cfg.pbpb);
	return HD_OK;
}

hd_status hd_edit_reserve(hd_pool *pool, uint64_t max_items, uint64_t max_list_entries, uint32_t max_edits) {
	if (!pool)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	return ws_reserve(pool, max_items, max_items, max_list_entries, max_edits);
}

hd_status hd_edit(hd_pool *pool, uint32_t root, const hd_edit_desc *edits, uint32_t n, uint32_t *out_root,
                  void *stream) {
	if (!pool || !out_root || (n && !edits))
		return HD_ERR_INVALID_ARG;
	*out_root = root;
	if (n == 0)
		return HD_OK;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	cudaStream_t st = (cudaStream_t)stream;
	hd_status s = ws_reserve(pool, 0, 0, 0, n);
	if (s)
		return s;
	return run_pass_sync(pool, edits, n, root, out_root, st);
}

hd_status hd_edit_async(hd_pool *pool, uint32_t root, const hd_edit_desc *d_edits, uint32_t n, uint32_t *d_out_root,
                        void *stream) {
	if (!pool || !d_out_root || !d_edits || n == 0)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	cudaStream_t st = (cudaStream_t)stream;
	hd_status s = launch_pass(pool, d_edits, n, root, nullptr, d_out_root, st, nullptr);
	if (s)
		return s;
	k_error_from_ws<<<1, 32, 0, st>>>(pool->P, pool->ws.d);
	pool->kernel_launches++;
	HD_TRY(cudaGetLastError());
	return hd_check(cudaEventRecord(pool->ws_free, st)); // hd_pool_get_error waits for this
}

hd_status hd_edit_async_droot(hd_pool *pool, const uint32_t *d_root, const hd_edit_desc *d_edits, uint32_t n,
                              uint32_t *d_out_root, void *stream) {
	if (!pool || !d_out_root || !d_edits || !d_root || n == 0)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	cudaStream_t st = (cudaStream_t)stream;
	hd_status s = launch_pass(pool, d_edits, n, kNull, d_root, d_out_root, st, nullptr);
	if (s)
		return s;
	k_error_from_ws<<<1, 32, 0, st>>>(pool->P, pool->ws.d);
	pool->kernel_launches++;
	HD_TRY(cudaGetLastError());
	return hd_check(cudaEventRecord(pool->ws_free, st)); // hd_pool_get_error waits for this
}

hd_status hd_edit_async_droot_hinted(hd_pool *pool, const uint32_t *d_root, const hd_edit_desc *d_edits,
                                     const hd_edit_desc *h_edits, uint32_t n, uint32_t *d_out_root, void *stream) {
	if (!pool || !d_out_root || !d_edits || !d_root || !h_edits || n == 0)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	cudaStream_t st = (cudaStream_t)stream;
	hd_status s = launch_pass(pool, d_edits, n, kNull, d_root, d_out_root, st, h_edits);
	if (s)
		return s;
	k_error_from_ws<<<1, 32, 0, st>>>(pool->P, pool->ws.d);
	pool->kernel_launches++;
	HD_TRY(cudaGetLastError());
	return hd_check(cudaEventRecord(pool->ws_free, st));
}

hd_status hd_edit_get_tuning(const hd_pool *pool, hd_tuning *out) {
	if (!pool || !out)
		return HD_ERR_INVALID_ARG;
	*out = pool->tune;
	return HD_OK;
}

hd_status hd_edit_set_tuning(hd_pool *pool, const hd_tuning *t) {
	if (!pool || !t || !t->expand_blocks_per_sm || !t->leaf_blocks_per_sm || !t->dedup_blocks_per_sm ||
	    !t->long_blocks_per_sm || !t->long_threshold || t->expand_blocks_per_sm > 64 || t->leaf_blocks_per_sm > 64 ||
	    t->dedup_blocks_per_sm > 64 || t->long_blocks_per_sm > 64 || t->leaf_compact > 1)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	pool->tune = *t;
	++pool->shape_gen;
	return HD_OK;
}

// Coordinate descent over the launch shape, one parameter at a time, each
// candidate timed (CUDA events, best of two) on the same pass from the same
// pool state (checkpoint before, rollback after every trial).
hd_status hd_edit_autotune(hd_pool *pool, uint32_t root, const hd_edit_desc *edits, uint32_t n, hd_tuning *out,
                           float *ms_before, float *ms_after) {
	if (!pool || !edits || !n)
		return HD_ERR_INVALID_ARG;
	hd_status s = hd_pool_checkpoint(pool);
	if (s)
		return s;
	uint32_t sized_root = kNull;
	s = hd_edit(pool, root, edits, n, &sized_root, nullptr); // sizes the workspace for this pass
	if (s)
		return s;
	HD_TRY(cudaSetDevice(pool->device));
	cudaStream_t st = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	hd_edit_desc *d_edits = nullptr;
	uint32_t *d_root = nullptr;
	auto cleanup = [&]() {
		if (d_edits)
			cudaFree(d_edits);
		if (d_root)
			cudaFree(d_root);
		if (e0)
			cudaEventDestroy(e0);
		if (e1)
			cudaEventDestroy(e1);
		if (st)
			cudaStreamDestroy(st);
	};
	if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
	    cudaEventCreate(&e1) != cudaSuccess || cudaMalloc(&d_edits, n * sizeof(hd_edit_desc)) != cudaSuccess ||
	    cudaMalloc(&d_root, 4) != cudaSuccess ||
	    cudaMemcpy(d_edits, edits, n * sizeof(hd_edit_desc), cudaMemcpyHostToDevice) != cudaSuccess) {
		cudaGetLastError();
		cleanup();
		return HD_ERR_CUDA;
	}
	auto trial = [&](const hd_tuning &t, float *ms) -> hd_status {
		float best = 1e30f;
		for (int rep = 0; rep < 2; ++rep) {
			hd_status r = hd_pool_rollback(pool, st);
			if (r)
				return r;
			{
				std::lock_guard<std::mutex> lk(pool->mtx);
				pool->tune = t;
				++pool->shape_gen;
			}
			if (cudaEventRecord(e0, st) != cudaSuccess)
				return HD_ERR_CUDA;
			r = hd_edit_async(pool, root, d_edits, n, d_root, st);
			if (r)
				return r;
			if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
				return HD_ERR_CUDA;
			uint32_t err = 0;
			if ((r = hd_pool_get_error(pool, &err)))
				return r;
			if (err) { // a pass that failed does not count (and must not happen: same pass as the sizing run)
				hd_pool_clear_error(pool);
				return HD_ERR_INTERNAL;
			}
			float ms_r = 0.0f;
			cudaEventElapsedTime(&ms_r, e0, e1);
			best = std::min(best, ms_r);
		}
		*ms = best;
		return HD_OK;
	};
	hd_tuning cur = pool->tune;
	float cur_ms = 0.0f;
	s = trial(cur, &cur_ms);
	const float start_ms = cur_ms;
	struct Knob {
		uint32_t hd_tuning::*field;
		std::vector<uint32_t> values;
	};
	const std::vector<Knob> knobs = {{&hd_tuning::leaf_compact, {0, 1}},
	                                 {&hd_tuning::long_threshold, {8, 16, 32, 64}},
	                                 {&hd_tuning::leaf_blocks_per_sm, {3, 6, 12, 24}},
	                                 {&hd_tuning::dedup_blocks_per_sm, {4, 8, 16, 32}},
	                                 {&hd_tuning::expand_blocks_per_sm, {4, 8, 16, 32}},
	                                 {&hd_tuning::long_blocks_per_sm, {2, 4, 8}}};
	for (const Knob &k : knobs) {
		if (s)
			break;
		for (uint32_t v : k.values) {
			if (v == cur.*(k.field))
				continue;
			hd_tuning t = cur;
			t.*(k.field) = v;
			float ms = 0.0f;
			if ((s = trial(t, &ms)))
				break;
			if (ms < cur_ms * 0.98f) { // keep a change only when it is clearly faster
				cur = t;
				cur_ms = ms;
			}
		}
	}
	{
		std::lock_guard<std::mutex> lk(pool->mtx);
		pool->tune = cur;
		++pool->shape_gen;
	}
	const hd_status rb = hd_pool_rollback(pool, st);
	if (!s)
		s = rb;
	cudaStreamSynchronize(st);
	cleanup();
	if (s)
		return s;
	if (out)
		*out = cur;
	if (ms_before)
		*ms_before = start_ms;
	if (ms_after)
		*ms_after = cur_ms;
	return HD_OK;
}

hd_status hd_edit_profile_begin(hd_pool *pool, uint32_t max_passes) {
	if (!pool)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	const uint64_t need = (uint64_t)max_passes * hd_prof_events_per_pass(pool->cfg.node_levels);
	while (pool->prof_events.size() < need) {
		cudaEvent_t e;
		HD_TRY(cudaEventCreate(&e));
		pool->prof_events.push_back(e);
	}
	pool->prof_passes = 0;
	pool->prof_max_passes = max_passes;
	return HD_OK;
}

hd_status hd_edit_profile_end(hd_pool *pool, float *out_ms, uint32_t *out_passes) {
	if (!pool || !out_ms)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	const uint32_t L = pool->cfg.node_levels, per = hd_prof_events_per_pass(L);
	for (uint32_t k = 0; k + 1 < per; ++k)
		out_ms[k] = 0.0f;
	for (uint32_t p = 0; p < pool->prof_passes; ++p) {
		cudaEvent_t *ev = pool->prof_events.data() + (uint64_t)p * per;
		HD_TRY(cudaEventSynchronize(ev[per - 1]));
		for (uint32_t k = 0; k + 1 < per; ++k) {
			float ms = 0.0f;
			HD_TRY(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
			out_ms[k] += ms;
		}
	}
	if (out_passes)
		*out_passes = pool->prof_passes;
	pool->prof_max_passes = 0;
	pool->prof_passes = 0;
	return HD_OK;
}

uint64_t hd_pool_kernel_launches(const hd_pool *pool) { return pool ? pool->kernel_launches.load() : 0; }

hd_status hd_pool_epoch(const hd_pool *pool, uint64_t *out) {
	if (!pool || !out)
		return HD_ERR_INVALID_ARG;
	*out = pool->epoch.load();
	return HD_OK;
}

hd_status hd_pool_checkpoint(hd_pool *pool) {
	if (!pool)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaDeviceSynchronize());
	const uint64_t slots = pool->P.index_mask + 1;
	if (!pool->ck_bucket_words) {
		if (cudaMalloc(&pool->ck_bucket_words, pool->total_buckets * 4) != cudaSuccess ||
		    cudaMalloc(&pool->ck_page_table, pool->total_pages * 4) != cudaSuccess ||
		    cudaMalloc(&pool->ck_counters, kCtrCount * 4) != cudaSuccess ||
		    cudaMalloc(&pool->ck_index, slots * 8) != cudaSuccess) {
			cudaGetLastError();
			cudaFree(pool->ck_bucket_words);
			cudaFree(pool->ck_page_table);
			cudaFree(pool->ck_counters);
			cudaFree(pool->ck_index);
			pool->ck_bucket_words = pool->ck_page_table = pool->ck_counters = nullptr;
			pool->ck_index = nullptr;
			return HD_ERR_POOL_OOM;
		}
	}
	HD_TRY(cudaMemcpy(pool->ck_bucket_words, pool->P.bucket_words, pool->total_buckets * 4, cudaMemcpyDeviceToDevice));
	HD_TRY(cudaMemcpy(pool->ck_page_table, pool->P.page_table, pool->total_pages * 4, cudaMemcpyDeviceToDevice));
	HD_TRY(cudaMemcpy(pool->ck_counters, pool->P.counters, kCtrCount * 4, cudaMemcpyDeviceToDevice));
	HD_TRY(cudaMemcpy(pool->ck_index, pool->P.index, slots * 8, cudaMemcpyDeviceToDevice));
	HD_TRY(cudaDeviceSynchronize()); // device-to-device copies return before they finish
	for (uint32_t l = 0; l < pool->cfg.node_levels; ++l)
		pool->ck_filled[l] = pool->P.cfg.filled[l];
	pool->has_checkpoint = true;
	return HD_OK;
}

hd_status hd_pool_rollback(hd_pool *pool, void *stream) {
	if (!pool)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	if (!pool->has_checkpoint)
		return HD_ERR_INVALID_ARG;
	++pool->epoch; // later passes write over the words dropped here
	HD_TRY(cudaSetDevice(pool->device));
	cudaStream_t st = (cudaStream_t)stream;
	HD_TRY(cudaStreamWaitEvent(st, pool->ws_free, 0));
	HD_TRY(cudaMemcpyAsync(pool->P.bucket_words, pool->ck_bucket_words, pool->total_buckets * 4,
	                       cudaMemcpyDeviceToDevice, st));
	HD_TRY(cudaMemcpyAsync(pool->P.page_table, pool->ck_page_table, pool->total_pages * 4, cudaMemcpyDeviceToDevice, st));
	HD_TRY(cudaMemcpyAsync(pool->P.counters, pool->ck_counters, kCtrCount * 4, cudaMemcpyDeviceToDevice, st));
	HD_TRY(cudaMemcpyAsync(pool->P.index, pool->ck_index, (pool->P.index_mask + 1) * 8, cudaMemcpyDeviceToDevice, st));
	bool filled_changed = false;
	for (uint32_t l = 0; l < pool->cfg.node_levels; ++l) {
		filled_changed = filled_changed || pool->P.cfg.filled[l] != pool->ck_filled[l];
		pool->P.cfg.filled[l] = pool->ck_filled[l];
	}
	if (filled_changed) // the filled pointers are kernel parameters of a captured pass graph
		++pool->shape_gen;
	HD_TRY(cudaEventRecord(pool->ws_free, st));
	return HD_OK;
}

hd_status hd_edit_last_counters(hd_pool *pool, uint64_t *items, uint64_t *candidates, uint64_t *candidate_words,
                                uint64_t *inserted, uint64_t *inserted_words) {
	if (!pool)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	std::vector<unsigned long long> c(kWsCtrCount);
	HD_TRY(cudaMemcpy(c.data(), pool->ws.d.ctr, kWsCtrCount * 8, cudaMemcpyDeviceToHost));
	for (uint32_t l = 0; l < pool->cfg.node_levels; ++l) {
		if (items)
			items[l] = c[kWsItems + l];
		if (candidates)
			candidates[l] = c[kWsCand + l];
		if (candidate_words)
			candidate_words[l] = c[kWsCandWords + l];
		if (inserted)
			inserted[l] = c[kWsIns + l];
		if (inserted_words)
			inserted_words[l] = c[kWsInsWords + l];
	}
	return HD_OK;
}

hd_status hd_edit_last_probe_stats(hd_pool *pool, uint64_t *probe_steps, uint64_t *max_probe, uint64_t *cas_retries) {
	if (!pool)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	std::vector<unsigned long long> c(kWsCtrCount);
	HD_TRY(cudaMemcpy(c.data(), pool->ws.d.ctr, kWsCtrCount * 8, cudaMemcpyDeviceToHost));
	if (probe_steps)
		*probe_steps = c[kWsProbeSteps];
	if (max_probe)
		*max_probe = c[kWsMaxProbe];
	if (cas_retries)
		*cas_retries = c[kWsCasRetry];
	return HD_OK;
}

hd_status hd_edit_last_leaf_work(hd_pool *pool, uint64_t *out) {
	if (!pool || !out)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	unsigned long long c[7];
	HD_TRY(cudaMemcpy(c, pool->ws.d.ctr + kWsLeafNodes, sizeof(c), cudaMemcpyDeviceToHost));
	for (int k = 0; k < 7; ++k)
		out[k] = c[k];
	return HD_OK;
}

hd_status hd_upsert(hd_pool *pool, uint32_t level, const uint32_t *words, const uint32_t *lens, uint32_t n,
                    uint32_t *out_ptrs) {
	if (!pool)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaMemset(pool->P.counters + kCtrError, 0, 4));
	return upsert_impl(pool, level, words, lens, n, out_ptrs);
}

hd_status hd_pool_read_bucket_words(const hd_pool *pool, uint32_t first, uint32_t count, uint32_t *out) {
	if (!pool || !out || (uint64_t)first + count > pool->total_buckets)
		return HD_ERR_INVALID_ARG;
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	HD_TRY(cudaMemcpy(out, pool->P.bucket_words + first, (uint64_t)count * 4, cudaMemcpyDeviceToHost));
	return HD_OK;
}

hd_status hd_pool_read_page_map(const hd_pool *pool, uint8_t *out) {
	if (!pool || !out)
		return HD_ERR_INVALID_ARG;
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	std::vector<uint32_t> pt(pool->total_pages);
	HD_TRY(cudaMemcpy(pt.data(), pool->P.page_table, pool->total_pages * 4, cudaMemcpyDeviceToHost));
	for (uint64_t i = 0; i < pool->total_pages; ++i)
		out[i] = pt[i] != kUnallocPage ? 1 : 0;
	return HD_OK;
}

hd_status hd_pool_read_pages(const hd_pool *pool, const uint32_t *page_ids, uint32_t n, uint32_t *out) {
	if (!pool || (n && (!page_ids || !out)))
		return HD_ERR_INVALID_ARG;
	if (!n)
		return HD_OK;
	for (uint32_t i = 0; i < n; ++i)
		if (page_ids[i] >= pool->total_pages)
			return HD_ERR_INVALID_ARG;
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaEventSynchronize(pool->ws_free));
	const uint64_t wp = 1ull << pool->P.cfg.wbpp;
	const uint32_t chunk = (uint32_t)std::max<uint64_t>(1, (64ull << 20) / (wp * 4));
	uint32_t *d_ids = nullptr, *d_buf = nullptr;
	HD_TRY(cudaMalloc(&d_ids, (uint64_t)chunk * 4));
	if (cudaMalloc(&d_buf, (uint64_t)chunk * wp * 4) != cudaSuccess) {
		cudaFree(d_ids);
		return HD_ERR_CUDA;
	}
	hd_status s = HD_OK;
	for (uint32_t b = 0; b < n && !s; b += chunk) {
		const uint32_t m = std::min(chunk, n - b);
		if (cudaMemcpy(d_ids, page_ids + b, m * 4ull, cudaMemcpyHostToDevice) != cudaSuccess) {
			s = HD_ERR_CUDA;
			break;
		}
		k_gather_pages<<<std::max(1u, std::min(ceil_div((uint64_t)m * wp, 256), 4096u)), 256>>>(pool->P, d_ids, m, d_buf);
		if (cudaMemcpy(out + (uint64_t)b * wp, d_buf, (uint64_t)m * wp * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
			s = HD_ERR_CUDA;
	}
	cudaFree(d_ids);
	cudaFree(d_buf);
	return s;
}

hd_status hd_pool_upload(hd_pool *pool, const uint32_t *bucket_words, const uint32_t *page_ids, uint32_t n_pages,
                         const uint32_t *page_words, const uint32_t *filled) {
	if (!pool || !bucket_words || (n_pages && (!page_ids || !page_words)))
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	HD_TRY(cudaDeviceSynchronize());
	if ((uint64_t)n_pages + 1 > pool->P.heap_pages)
		return HD_ERR_POOL_OOM;
	const uint64_t wp = 1ull << pool->P.cfg.wbpp;
	const uint64_t wpb = 1ull << (pool->P.cfg.wbpp + pool->P.cfg.pbpb);
	for (uint64_t b = 0; b < pool->total_buckets; ++b)
		if (bucket_words[b] > wpb)
			return HD_ERR_INVALID_ARG;
	std::vector<uint32_t> pt(pool->total_pages, kUnallocPage);
	for (uint32_t i = 0; i < n_pages; ++i) {
		if (page_ids[i] >= pool->total_pages)
			return HD_ERR_INVALID_ARG;
		pt[page_ids[i]] = pool->P.identity ? page_ids[i] : i + 1;
	}
	++pool->epoch; // every word is replaced
	HD_TRY(cudaMemcpy(pool->P.bucket_words, bucket_words, pool->total_buckets * 4, cudaMemcpyHostToDevice));
	HD_TRY(cudaMemcpy(pool->P.page_table, pt.data(), pool->total_pages * 4, cudaMemcpyHostToDevice));
	HD_TRY(cudaMemset(pool->P.heap, 0, (uint64_t)pool->P.heap_pages * wp * 4));
	for (uint32_t i = 0; i < n_pages; ++i) { // one copy per page: the layout differs per mode
		const uint64_t phys = pt[page_ids[i]];
		HD_TRY(cudaMemcpyAsync(pool->P.heap + phys * wp, page_words + (uint64_t)i * wp, wp * 4, cudaMemcpyHostToDevice));
	}
	HD_TRY(cudaDeviceSynchronize());
	uint32_t ctr0[kCtrCount] = {n_pages + 1u, 0u, 0u, 0u};
	HD_TRY(cudaMemcpy(pool->P.counters, ctr0, sizeof(ctr0), cudaMemcpyHostToDevice));
	hd_status s = hd_rebuild_index(pool, nullptr);
	if (s)
		return s;
	if (filled) {
		for (uint32_t l = 0; l < pool->cfg.node_levels; ++l)
			pool->P.cfg.filled[l] = filled[l];
		++pool->shape_gen;
		return HD_OK;
	}
	return make_filled(pool);
}

hd_status hd_query(hd_pool *pool, uint32_t root, const uint32_t *xyz, uint32_t n, uint8_t *out, void *stream) {
	if (!pool || (n && (!xyz || !out)))
		return HD_ERR_INVALID_ARG;
	if (!n)
		return HD_OK;
	std::lock_guard<std::mutex> lk(pool->mtx);
	HD_TRY(cudaSetDevice(pool->device));
	cudaStream_t st = (cudaStream_t)stream;
	uint32_t *d_xyz = nullptr;
	uint8_t *d_out = nullptr;
	HD_TRY(cudaMalloc(&d_xyz, n * 12ull));
	if (cudaMalloc(&d_out, n) != cudaSuccess) {
		cudaFree(d_xyz);
		return HD_ERR_CUDA;
	}
	hd_status s = HD_OK;
	if (cudaStreamWaitEvent(st, pool->ws_free, 0) != cudaSuccess ||
	    cudaMemcpyAsync(d_xyz, xyz, n * 12ull, cudaMemcpyHostToDevice, st) != cudaSuccess)
		s = HD_ERR_CUDA;
	if (!s) {
		k_query<<<std::max(1u, std::min(ceil_div(n, 256), 8192u)), 256, 0, st>>>(pool->P, root, d_xyz, n, d_out);
		if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(out, d_out, n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
		    cudaStreamSynchronize(st) != cudaSuccess)
			s = HD_ERR_CUDA;
	}
	cudaFree(d_xyz);
	cudaFree(d_out);
	return s;
}

uint64_t hd_count_voxel_edits(const hd_edit_desc *edits, uint32_t n, uint32_t res) {
	std::unordered_map<uint64_t, uint64_t> memo; // unclipped spheres depend on r2 only
	uint64_t total = 0;
	for (uint32_t i = 0; i < n; ++i) {
		const hd_edit_desc &e = edits[i];
		if (e.shape == HD_SHAPE_AABB) {
			uint64_t c = 1;
			for (int a = 0; a < 3; ++a) {
				uint64_t lo = std::min<uint64_t>(e.p0[a], res), hi = std::min<uint64_t>(e.p1[a], res);
				c *= hi > lo ? hi - lo : 0;
			}
			total += c;
			continue;
		}
		const int64_t r = isqrt64(e.r2);
		bool inside = true;
		for (int a = 0; a < 3; ++a)
			inside = inside && (int64_t)e.p0[a] - r >= 0 && (int64_t)e.p0[a] + r < (int64_t)res;
		if (inside) {
			auto it = memo.find(e.r2);
			if (it == memo.end())
				it = memo.emplace(e.r2, sphere_count(r, r, r, e.r2, 2 * r + 1)).first;
			total += it->second;
		} else
			total += sphere_count(e.p0[0], e.p0[1], e.p0[2], e.r2, res);
	}
	return total;
}

} // extern "C"
