// hd_noalloc.cu -- find-or-insert of caller nodes without any allocation.
//
// Some callers cannot call cudaMalloc at the moment they want to insert
// nodes: applications that hand the whole device memory to their own
// allocator up front (as the reference renderer does with its sparse Vulkan
// buffers), or latency-bound edit loops that must not take the implicit device
// synchronisation a cudaMalloc/cudaFree can cause.  hd_upsert_noalloc serves
// them: it runs the same dedup kernel as hd_upsert (k_dedup), but the
// per-node scratch that kernel needs lives in the file-scope device array
// g_upsert_scratch below instead of the pool's cudaMalloc'ed workspace.
//
// Limits and sharing:
//   * at most kNoAllocMaxNodes nodes per call (larger calls are rejected with
//     HD_ERR_INVALID_ARG before anything runs);
//   * the array is static device memory: every GPU that loads this library
//     holds its kScratchBytes until the process exits;
//   * every call on every pool of a device shares the one array and it keeps
//     the previous call's contents; the counters that must start at zero are
//     cleared at the start of each call, and calls that overlap on the GPU
//     (different streams without ordering between them) race on the array.
//   * the device address of the array is looked up once per device, on the
//     first call on that device (cudaGetSymbolAddress with the device
//     current); make that first call before any stream capture.
#include "hd_internal.h"
#include "hd_kernels.cuh"

#include <cstdio>
#include <mutex>

using namespace hd;

namespace {

constexpr uint32_t kNoAllocMaxNodes = 65536;
constexpr uint32_t kCtrWords = kWsCtrCount;
// per node: res, parent (2 words) + cnew and bchild (16 words)
constexpr size_t kNodeScratchWords = 18;
constexpr size_t kScratchBytes =
    kCtrWords * sizeof(unsigned long long) + (size_t)kNoAllocMaxNodes * kNodeScratchWords * sizeof(uint32_t);

static __device__ __align__(256) unsigned char g_upsert_scratch[kScratchBytes];

// per-device address of g_upsert_scratch, filled on the first call on that device
constexpr int kMaxDevices = 64;
std::mutex g_addr_mutex;
void *g_addr[kMaxDevices] = {};

hd_status scratch_address(int device, unsigned char **out) {
	if (device < 0 || device >= kMaxDevices)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(g_addr_mutex);
	if (!g_addr[device]) {
		void *p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_upsert_scratch);
		if (e != cudaSuccess) {
			fprintf(stderr, "hashdag_gb300: cudaGetSymbolAddress(g_upsert_scratch) failed: %s\n", cudaGetErrorString(e));
			return HD_ERR_CUDA;
		}
		g_addr[device] = p;
	}
	*out = static_cast<unsigned char *>(g_addr[device]);
	return HD_OK;
}

// Workspace view of the scratch: counters first, then the per-node arrays.
Workspace scratch_workspace(unsigned char *base, uint32_t n, bool leaf) {
	Workspace W{};
	W.ctr = reinterpret_cast<unsigned long long *>(base);
	uint32_t *w = reinterpret_cast<uint32_t *>(base + kCtrWords * sizeof(unsigned long long));
	Items it{};
	it.cap = n;
	it.res = w;
	it.parent = w + (size_t)kNoAllocMaxNodes;
	uint32_t *tail = w + 2 * (size_t)kNoAllocMaxNodes; // 16 words per node, 256-byte aligned offset
	if (leaf) {
		W.leaf = it;
		W.leaf_new = reinterpret_cast<u64 *>(tail);
	} else {
		W.inner = it;
		W.cnew = tail;
		W.bchild = tail + 8 * (size_t)kNoAllocMaxNodes;
	}
	W.n_edits = 0;
	W.long_threshold = 16;
	return W;
}

// Loads the caller's nodes into the scratch.  Inner level: 8 child pointers per
// node (Null = 0xFFFFFFFF), in child order.  Leaf level: 2 words per node.
// An inner node with no child is an invalid argument (hd_upsert rejects it on
// the host): it fails the whole call through the workspace error word, so the
// dedup launch inserts nothing and every result becomes Null.
__global__ void k_noalloc_load(Workspace W, const uint32_t *nodes, uint32_t n, uint32_t level, uint32_t leaf) {
	const u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
	if (i == 0)
		W.ctr[kWsItems + level] = n;
	if (i >= n)
		return;
	if (leaf) {
		W.leaf_new[i] = (u64)nodes[2 * i] | ((u64)nodes[2 * i + 1] << 32);
		W.leaf.parent[i] = kNull;
	} else {
		u32 any = 0;
		for (int c = 0; c < 8; ++c) {
			const u32 v = nodes[i * 8 + c];
			W.cnew[i * 8 + c] = v;
			// the base children differ from the new ones in every slot, so the
			// dedup launch always builds and looks up the node; it never takes
			// its "no child changed" branch, which reads a base node this
			// scratch does not have
			W.bchild[i * 8 + c] = v ^ 1u;
			any |= v != kNull ? 1u : 0u;
		}
		if (!any)
			atomicCAS(&W.ctr[kWsError], 0ull, (unsigned long long)kErrInvalidRoot);
		W.inner.parent[i] = kNull;
	}
}

// Copies the results out.  A failed call (its own workspace error, or the
// pool's sticky error, which the dedup launch may have just set) writes Null
// for every node, so no pointer of an earlier call left in the shared scratch
// can come back; the workspace error also becomes the pool's error.
__global__ void k_noalloc_store(DevPool P, Workspace W, uint32_t n, uint32_t leaf, uint32_t *out) {
	const u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
	const unsigned long long ws_err = *(volatile unsigned long long *)&W.ctr[kWsError];
	if (i == 0 && ws_err)
		set_error(&P.counters[kCtrError], (u32)ws_err);
	const bool failed = ws_err != 0 || *(volatile u32 *)&P.counters[kCtrError] != 0;
	if (i < n)
		out[i] = failed ? kNull : (leaf ? W.leaf.res[i] : W.inner.res[i]);
}

} // namespace

extern "C" hd_status hd_upsert_noalloc(hd_pool *pool, uint32_t level, const uint32_t *d_nodes, uint32_t n,
                                       uint32_t *d_out_ptrs, void *stream) {
	if (!pool || level >= pool->cfg.node_levels || (n && (!d_nodes || !d_out_ptrs)))
		return HD_ERR_INVALID_ARG;
	if (n > kNoAllocMaxNodes) {
		fprintf(stderr, "hashdag_gb300: hd_upsert_noalloc takes at most %u nodes per call (got %u)\n",
		        kNoAllocMaxNodes, n);
		return HD_ERR_INVALID_ARG;
	}
	if (n == 0)
		return HD_OK;
	std::lock_guard<std::mutex> lk(pool->mtx);
	if (cudaSetDevice(pool->device) != cudaSuccess)
		return HD_ERR_CUDA;
	unsigned char *base = nullptr;
	hd_status s = scratch_address(pool->device, &base);
	if (s)
		return s;
	const bool leaf = level == pool->cfg.node_levels - 1;
	Workspace W = scratch_workspace(base, n, leaf);
	cudaStream_t st = (cudaStream_t)stream;
	const uint32_t grid = (n + kBlock - 1) / kBlock;
	if (cudaStreamWaitEvent(st, pool->ws_free, 0) != cudaSuccess ||
	    cudaMemsetAsync(W.ctr, 0, kCtrWords * sizeof(unsigned long long), st) != cudaSuccess)
		return HD_ERR_CUDA;
	k_noalloc_load<<<grid, kBlock, 0, st>>>(W, d_nodes, n, level, leaf ? 1u : 0u);
	if (leaf)
		k_dedup<true><<<grid, kBlock, 0, st>>>(pool->P, W, level, 0u);
	else
		k_dedup<false><<<grid, kBlock, 0, st>>>(pool->P, W, level, 0u);
	k_finish<<<1, 32, 0, st>>>(pool->P, W, nullptr);
	k_noalloc_store<<<grid, kBlock, 0, st>>>(pool->P, W, n, leaf ? 1u : 0u, d_out_ptrs);
	if (cudaGetLastError() != cudaSuccess || cudaEventRecord(pool->ws_free, st) != cudaSuccess)
		return HD_ERR_CUDA;
	pool->kernel_launches += 4;
	return HD_OK;
}
