// hd_internal.h -- host-side state of a device node pool (shared by the .cu files).
#pragma once

#include "hd_device.cuh"

#include <atomic>
#include <mutex>
#include <vector>

struct hd_ws_host {
	hd::Workspace d{};          // device view handed to kernels
	std::vector<void *> allocs; // everything cudaMalloc'ed for the workspace
	hd_edit_desc *edits = nullptr;
	uint32_t edit_cap = 0;
	unsigned long long *ctr_host = nullptr; // pinned copy of the counters
};

struct hd_pool {
	int device = 0;
	int num_sms = 152;
	hd_config cfg{};
	hd::DevPool P{};
	uint64_t total_buckets = 0, total_pages = 0;
	uint32_t *d_out_root = nullptr; // device word for synchronous calls
	uint32_t *h_small = nullptr;    // pinned scratch (root, error)
	cudaEvent_t ws_free = nullptr;  // orders passes that share the workspace
	hd_ws_host ws;
	std::mutex mtx;
	uint64_t last_items[HD_MAX_LEVELS] = {}, last_cand[HD_MAX_LEVELS] = {}, last_ins[HD_MAX_LEVELS] = {};
	std::atomic<uint64_t> kernel_launches{0}; // kernels launched by this pool since creation (any thread)
	hd_tuning tune{8, 12, 32, 4, 16, 1};      // launch shape of the batched pass (the autotuner's pick on the benchmark)
	// CUDA graph of the multi-kernel pass of hd_edit, valid for one workspace
	// allocation and launch shape (shape_gen changes with either)
	uint64_t shape_gen = 0, graph_gen = ~0ull;
	cudaGraphExec_t pass_graph = nullptr;
	uint32_t pass_graph_kernels = 0;
	cudaStream_t capture_stream = nullptr;
	// phase timing: one set of events per profiled pass
	std::vector<cudaEvent_t> prof_events;
	uint32_t prof_passes = 0, prof_max_passes = 0;
	// checkpoint: device copies of the pool's mutable state
	uint32_t *ck_bucket_words = nullptr, *ck_page_table = nullptr, *ck_counters = nullptr;
	unsigned long long *ck_index = nullptr;
	uint32_t ck_filled[HD_MAX_LEVELS] = {};
	bool has_checkpoint = false;
	// generation of the committed words: bumped by every call that rewrites or
	// drops words already in the pool (hd_gc, hd_pool_rollback, hd_pool_upload);
	// between two equal values the pool only appended (hd_pool_epoch)
	std::atomic<uint64_t> epoch{0};
};

// events per profiled pass: start, after expand, after leaf, after the dedup launch
// of every level (1 per level), after finish
inline uint32_t hd_prof_events_per_pass(uint32_t L) { return 3u + L + 1u; }

// hd_engine.cu
hd_status hd_check(cudaError_t e);
hd_status hd_rebuild_index(hd_pool *pool, cudaStream_t st); // dedup index from the bucket contents (synchronous)
hd_status hd_remake_filled(hd_pool *pool); // filled-node pointers found or inserted again
// hd_trace.cu (no wait for edit passes on other streams; the caller orders)
hd_status hd_launch_pinhole(hd_pool *pool, uint32_t root, const hd_camera *d_cams, uint32_t n_cameras, uint32_t width,
                            uint32_t height, hd_hit *d_out, uint64_t *d_counters, cudaStream_t st);
hd_status hd_launch_pinhole_stackless(hd_pool *pool, uint32_t root, const hd_camera *d_cams, uint32_t n_cameras,
                                      uint32_t width, uint32_t height, hd_hit *d_out, uint64_t *d_counters,
                                      cudaStream_t st);
hd_status hd_launch_rays(hd_pool *pool, uint32_t root, const float *d_o, const float *d_d, uint32_t n, hd_hit *d_out,
                         cudaStream_t st);
void hd_grid_for_levels(const hd_pool *pool, const hd_edit_desc *host_edits, uint32_t n, uint32_t *grid_per_level);
