// hd_gc.cu -- garbage collection of a device pool: mark from the roots, then
// compact every level bottom-up into the layout the reference's collector
// writes (include/hashdag/NodePoolThreadedGC.hpp:29-403, ThreadedGC run by one
// worker), so a collected pool is word-identical to the reference's.
//
// Steps (all on the device; the pool is only written once every step that can
// fail has succeeded):
//   1. mark: a bitmap over the pool's word space, one bit per live node start.
//      Roots (the filled root first, :357-369) are set on the host side; each
//      level's live nodes then set their children's bits (:29-103).  Only bits
//      inside a level's word range are read while that level is expanded.
//   2. rank: popcount prefix of the bitmap; the live list G holds every live
//      pointer in ascending order (= old bucket, then old offset: the order the
//      reference sorts each bucket's list in, :36-37).  rank(ptr) indexes G.
//   3. leaves (L-1): each bucket keeps its leaves, re-appended from offset 0 in
//      rank order with the page padding rule (:223-265).
//   4. inner levels L-2..0: children remapped through the new pointers of the
//      level below, node re-hashed, new bucket = hash & mask; a stable radix
//      sort by new bucket keeps rank order inside a bucket, i.e. the
//      reference's append order into its bucket caches (:105-171); one thread
//      per bucket lays its run out with the padding rule (:154-163).
//   5. physical pages: each bucket needs ceil(words / words_per_page) pages;
//      paged heaps renumber them densely (page 0 stays the zero page), an
//      identity heap keeps virtual = physical.  Then the heap is cleared and
//      every live node written at its new place, bucket word counts set, the
//      dedup index rebuilt and the filled nodes found again (:378-381).
// Radix sort and prefix sums come from CUB (library primitives, not the edit
// path).
#include "hd_internal.h"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstdio>
#include <vector>

using namespace hd;

namespace {

constexpr u32 kGcBlock = 256;
constexpr u32 kGcErrPointer = 1u, kGcErrBucket = 2u;

__device__ __forceinline__ u32 rank_of(const u32 *bm, const u32 *prefix, u64 ptr) {
	const u64 w = ptr >> 5;
	const u32 b = (u32)(ptr & 31u);
	return prefix[w] + (b ? __popc(bm[w] & ((1u << b) - 1u)) : 0u);
}

__device__ __forceinline__ u32 grid_stride_begin() { return blockIdx.x * blockDim.x + threadIdx.x; }

// A pointer that names a node start inside level `l`'s bucket range and below
// its bucket's word count.
__device__ __forceinline__ bool valid_node(const DevPool &P, u32 l, u64 ptr) {
	const u32 wbpb = P.cfg.wbpp + P.cfg.pbpb;
	const u64 b = ptr >> wbpb;
	const u64 lo = P.cfg.bucket_base[l], hi = lo + (1ull << P.cfg.bucket_bits[l]);
	if (b < lo || b >= hi)
		return false;
	if ((ptr & ((1ull << wbpb) - 1u)) >= P.bucket_words[b])
		return false;
	const u32 phys = P.page_table[ptr >> P.cfg.wbpp];
	return phys != kUnallocPage && !page_lost(P, phys);
}

__global__ void k_gc_roots(DevPool P, u32 *bm, const u32 *roots, u32 n, u32 *err) {
	for (u32 i = grid_stride_begin(); i < n; i += gridDim.x * blockDim.x) {
		const u32 r = roots[i];
		if (r == kNull)
			continue;
		if (!valid_node(P, 0, r)) {
			atomicOr(err, kGcErrPointer);
			continue;
		}
		atomicOr(&bm[r >> 5], 1u << (r & 31u));
	}
}

// Live nodes of level l (bits of [lo, hi)) set the bits of their children.
__global__ void k_gc_mark(DevPool P, u32 *bm, u32 l, u64 lo, u64 hi, u32 *err) {
	const u64 w_lo = lo >> 5, w_hi = (hi + 31) >> 5;
	const u64 stride = (u64)gridDim.x * blockDim.x;
	for (u64 w = w_lo + grid_stride_begin(); w < w_hi; w += stride) {
		u32 bits = bm[w];
		const u64 base = w << 5;
		if (base < lo)
			bits &= ~0u << (u32)(lo - base);
		if (base + 32 > hi)
			bits &= (u32)((1ull << (u32)(hi - base)) - 1u);
		while (bits) {
			const u32 b = __ffs(bits) - 1u;
			bits &= bits - 1u;
			const u32 ptr = (u32)(base + b);
			const u32 *p = node_addr(P, ptr);
			const u32 m = p[0];
			if (m == 0u || m > 0xFFu) {
				atomicOr(err, kGcErrPointer);
				continue;
			}
			const u32 nc = __popc(m);
			for (u32 k = 0; k < nc; ++k) {
				const u32 c = p[1 + k];
				if (!valid_node(P, l + 1, c)) {
					atomicOr(err, kGcErrPointer);
					continue;
				}
				atomicOr(&bm[c >> 5], 1u << (c & 31u));
			}
		}
	}
}

__global__ void k_gc_popc(const u32 *bm, u64 nbw, u32 *counts) {
	const u64 stride = (u64)gridDim.x * blockDim.x;
	for (u64 w = grid_stride_begin(); w < nbw; w += stride)
		counts[w] = __popc(bm[w]);
}

__global__ void k_gc_list(const u32 *bm, const u32 *prefix, u64 nbw, u32 *G) {
	const u64 stride = (u64)gridDim.x * blockDim.x;
	for (u64 w = grid_stride_begin(); w < nbw; w += stride) {
		u32 bits = bm[w];
		u32 r = prefix[w];
		while (bits) {
			const u32 b = __ffs(bits) - 1u;
			bits &= bits - 1u;
			G[r++] = (u32)((w << 5) + b);
		}
	}
}

__global__ void k_gc_ranks(const u32 *bm, const u32 *prefix, const u64 *ptrs, u32 n, u32 *out) {
	for (u32 i = grid_stride_begin(); i < n; i += gridDim.x * blockDim.x)
		out[i] = rank_of(bm, prefix, ptrs[i]);
}

// Next offset for a node of `len` words at bucket offset `off` (no straddling
// a page: NodePool.hpp:134-157 append_node, NodePoolThreadedGC.hpp:154-163).
__device__ __forceinline__ u32 place(u32 off, u32 len, u32 wbpp) {
	const u32 wp = 1u << wbpp;
	return (off & (wp - 1u)) + len > wp ? ((off >> wbpp) + 1u) << wbpp : off;
}

// Leaf level: thread per bucket, its live leaves in rank order from offset 0.
__global__ void k_gc_leaf_layout(DevPool P, const u32 *bm, const u32 *prefix, const u32 *G, u32 g0, u32 *newp,
                                 u32 *words, u32 *new_bw, u32 *err) {
	const u32 l = P.cfg.L - 1, wbpb = P.cfg.wbpp + P.cfg.pbpb;
	const u32 nb = 1u << P.cfg.bucket_bits[l], base = P.cfg.bucket_base[l];
	const u64 wpb = 1ull << wbpb;
	for (u32 k = grid_stride_begin(); k < nb; k += gridDim.x * blockDim.x) {
		const u32 b = base + k;
		const u32 r0 = rank_of(bm, prefix, (u64)b << wbpb), r1 = rank_of(bm, prefix, (u64)(b + 1) << wbpb);
		u32 off = 0;
		for (u32 r = r0; r < r1; ++r) {
			const u32 *p = node_addr(P, G[r]);
			off = place(off, 2u, P.cfg.wbpp);
			if ((u64)off + 2u > wpb) {
				atomicOr(err, kGcErrBucket);
				break;
			}
			newp[r] = (b << wbpb) | off;
			words[2ull * (r - g0)] = p[0];
			words[2ull * (r - g0) + 1] = p[1];
			off += 2u;
		}
		new_bw[b] = off;
	}
}

// Inner level l, thread per live node j (rank g0 + j): children remapped,
// words staged, new bucket key.
__global__ void k_gc_inner_prep(DevPool P, const u32 *bm, const u32 *prefix, const u32 *G, u32 g0, u32 n, u32 l,
                                const u32 *newp, u32 *words, u32 *lens, u32 *keys, u32 *vals) {
	const u32 key_mask = (1u << P.cfg.bucket_bits[l]) - 1u;
	const bool zero_hash = P.cfg.hasher == HD_HASHER_ZERO;
	for (u32 j = grid_stride_begin(); j < n; j += gridDim.x * blockDim.x) {
		const u32 *p = node_addr(P, G[g0 + j]);
		const u32 m = p[0], nc = __popc(m);
		u32 *w = words + 9ull * j;
		w[0] = m;
		Murmur mm;
		mm.add(m);
		for (u32 k = 0; k < nc; ++k) {
			const u32 c = newp[rank_of(bm, prefix, p[1 + k])];
			w[1 + k] = c;
			mm.add(c);
		}
		lens[j] = nc + 1u;
		keys[j] = zero_hash ? 0u : (mm.finish(nc + 1u) & key_mask);
		vals[j] = j;
	}
}

// Run boundaries of the sorted keys: bucket key k owns sorted positions [begin[k], end[k]).
__global__ void k_gc_runs(const u32 *keys, u32 n, u32 *begin, u32 *end) {
	for (u32 j = grid_stride_begin(); j < n; j += gridDim.x * blockDim.x) {
		const u32 k = keys[j];
		if (j == 0 || keys[j - 1] != k)
			begin[k] = j;
		if (j + 1 == n || keys[j + 1] != k)
			end[k] = j + 1;
	}
}

// Thread per bucket of level l: lays out its run (stable rank order).
__global__ void k_gc_inner_layout(DevPool P, u32 l, const u32 *begin, const u32 *end, const u32 *vals, const u32 *lens,
                                  u32 g0, u32 *newp, u32 *new_bw, u32 *err) {
	const u32 wbpb = P.cfg.wbpp + P.cfg.pbpb, nb = 1u << P.cfg.bucket_bits[l], base = P.cfg.bucket_base[l];
	const u64 wpb = 1ull << wbpb;
	for (u32 k = grid_stride_begin(); k < nb; k += gridDim.x * blockDim.x) {
		u32 off = 0;
		for (u32 j = begin[k]; j < end[k]; ++j) {
			const u32 i = vals[j], len = lens[i];
			off = place(off, len, P.cfg.wbpp);
			if ((u64)off + len > wpb) { // the bucket cannot hold its nodes
				atomicOr(err, kGcErrBucket);
				break;
			}
			newp[g0 + i] = ((base + k) << wbpb) | off;
			off += len;
		}
		new_bw[base + k] = off;
	}
}

__global__ void k_gc_page_counts(const u32 *new_bw, u32 total_buckets, u32 wbpp, u32 *pages) {
	for (u32 b = grid_stride_begin(); b < total_buckets; b += gridDim.x * blockDim.x)
		pages[b] = (new_bw[b] + (1u << wbpp) - 1u) >> wbpp;
}

__global__ void k_gc_page_table(DevPool P, u32 total_buckets, const u32 *pages, const u32 *page_base) {
	for (u32 b = grid_stride_begin(); b < total_buckets; b += gridDim.x * blockDim.x)
		for (u32 j = 0; j < pages[b]; ++j) {
			const u32 vp = (b << P.cfg.pbpb) | j;
			P.page_table[vp] = P.identity ? vp : 1u + page_base[b] + j;
		}
}

// Writable address of a node through the (new) page table.
__device__ __forceinline__ u32 *node_addr_w(const DevPool &P, u32 ptr) {
	if (P.identity)
		return P.heap + ptr;
	const u32 phys = P.page_table[ptr >> P.cfg.wbpp];
	return P.heap + ((u64)phys << P.cfg.wbpp) + (ptr & (wpp(P.cfg) - 1u));
}

__global__ void k_gc_write(DevPool P, const u32 *newp, u32 g0, u32 n, const u32 *words, const u32 *lens, u32 stride_w) {
	for (u32 j = grid_stride_begin(); j < n; j += gridDim.x * blockDim.x) {
		u32 *dst = node_addr_w(P, newp[g0 + j]);
		const u32 len = lens ? lens[j] : 2u;
		const u32 *src = words + (u64)stride_w * j;
		for (u32 k = 0; k < len; ++k)
			dst[k] = src[k];
	}
}

__global__ void k_gc_remap_roots(const u32 *bm, const u32 *prefix, const u32 *newp, u32 *roots, u32 n) {
	for (u32 i = grid_stride_begin(); i < n; i += gridDim.x * blockDim.x)
		if (roots[i] != kNull)
			roots[i] = newp[rank_of(bm, prefix, roots[i])];
}

// Stream-ordered scratch of one collection (no device-wide synchronisation
// from allocation or release), released together on the collection's stream.
struct GcMem {
	cudaStream_t st;
	std::vector<void *> ptrs;
	explicit GcMem(cudaStream_t s) : st(s) {}
	template <typename T> hd_status alloc(T **p, uint64_t n) {
		void *q = nullptr;
		if (cudaMallocAsync(&q, std::max<uint64_t>(n, 1) * sizeof(T), st) != cudaSuccess) {
			cudaGetLastError();
			return HD_ERR_POOL_OOM;
		}
		ptrs.push_back(q);
		*p = static_cast<T *>(q);
		return HD_OK;
	}
	~GcMem() {
		for (void *p : ptrs)
			cudaFreeAsync(p, st);
		cudaStreamSynchronize(st);
	}
};

uint32_t grid_for(uint64_t n, int sms) {
	return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n + kGcBlock - 1) / kGcBlock, (uint64_t)sms * 16));
}

#define GC_TRY(x)                                                                                                   \
	do {                                                                                                            \
		hd_status s_ = (x);                                                                                         \
		if (s_)                                                                                                     \
			return s_;                                                                                              \
	} while (0)
#define GC_CUDA(x) GC_TRY(hd_check(x))

hd_status gc_impl(hd_pool *pool, uint32_t *roots, uint32_t n_roots, hd_gc_stats *stats, cudaStream_t st) {
	const hd_config &cfg = pool->cfg;
	const uint32_t L = cfg.node_levels, wbpb = cfg.word_bits_per_page + cfg.page_bits_per_bucket;
	const uint64_t total_words = pool->total_buckets << wbpb, nbw = (total_words + 31) / 32;
	const int sms = pool->num_sms;
	DevPool P = pool->P;
	GcMem mem(st);
	u32 *bm, *counts, *prefix, *err;
	GC_TRY(mem.alloc(&bm, nbw + 1));
	GC_TRY(mem.alloc(&counts, nbw + 1));
	GC_TRY(mem.alloc(&prefix, nbw + 1));
	GC_TRY(mem.alloc(&err, 1));
	GC_CUDA(cudaMemsetAsync(bm, 0, (nbw + 1) * 4, st));
	GC_CUDA(cudaMemsetAsync(err, 0, 4, st));

	// 1. mark
	std::vector<uint32_t> r0;
	if (P.cfg.filled[0] != kNull)
		r0.push_back(P.cfg.filled[0]);
	for (uint32_t i = 0; i < n_roots; ++i)
		if (roots[i] != kNull)
			r0.push_back(roots[i]);
	u32 *d_roots;
	GC_TRY(mem.alloc(&d_roots, r0.size() + n_roots));
	GC_CUDA(cudaMemcpyAsync(d_roots, r0.data(), r0.size() * 4, cudaMemcpyHostToDevice, st));
	k_gc_roots<<<grid_for(r0.size(), sms), kGcBlock, 0, st>>>(P, bm, d_roots, (u32)r0.size(), err);
	std::vector<uint64_t> lvl_lo(L + 1);
	for (uint32_t l = 0; l < L; ++l)
		lvl_lo[l] = (uint64_t)P.cfg.bucket_base[l] << wbpb;
	lvl_lo[L] = total_words;
	for (uint32_t l = 0; l + 1 < L; ++l)
		k_gc_mark<<<grid_for((lvl_lo[l + 1] - lvl_lo[l]) / 32 + 1, sms), kGcBlock, 0, st>>>(P, bm, l, lvl_lo[l],
		                                                                                     lvl_lo[l + 1], err);
	GC_CUDA(cudaGetLastError());
	uint32_t h_err = 0;
	GC_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, st));
	GC_CUDA(cudaStreamSynchronize(st));
	if (h_err) {
		fprintf(stderr, "hashdag_gb300: hd_gc: a root or a child pointer does not name a node of its level\n");
		return HD_ERR_INVALID_ARG;
	}

	// 2. ranks and the live list
	k_gc_popc<<<grid_for(nbw + 1, sms), kGcBlock, 0, st>>>(bm, nbw + 1, counts);
	size_t tmp_bytes = 0;
	GC_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, counts, prefix, (int)(nbw + 1), st));
	unsigned char *tmp;
	GC_TRY(mem.alloc(&tmp, tmp_bytes));
	GC_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, counts, prefix, (int)(nbw + 1), st));
	u64 *d_lvl;
	u32 *d_rank;
	GC_TRY(mem.alloc(&d_lvl, L + 1));
	GC_TRY(mem.alloc(&d_rank, L + 1));
	GC_CUDA(cudaMemcpyAsync(d_lvl, lvl_lo.data(), (L + 1) * 8, cudaMemcpyHostToDevice, st));
	k_gc_ranks<<<1, 32, 0, st>>>(bm, prefix, d_lvl, L + 1, d_rank);
	std::vector<uint32_t> g(L + 1);
	GC_CUDA(cudaMemcpyAsync(g.data(), d_rank, (L + 1) * 4, cudaMemcpyDeviceToHost, st));
	GC_CUDA(cudaStreamSynchronize(st));
	const uint64_t live = g[L];
	u32 *G, *newp;
	GC_TRY(mem.alloc(&G, live));
	GC_TRY(mem.alloc(&newp, live));
	k_gc_list<<<grid_for(nbw, sms), kGcBlock, 0, st>>>(bm, prefix, nbw, G);

	// 3.-4. new layout, level by level from the leaves up
	uint64_t max_n = 0, max_nb = 0;
	for (uint32_t l = 0; l < L; ++l) {
		max_n = std::max<uint64_t>(max_n, g[l + 1] - g[l]);
		max_nb = std::max<uint64_t>(max_nb, 1ull << cfg.bucket_bits_each_level[l]);
	}
	u32 *new_bw, *keys, *keys_out, *vals, *vals_out, *run_b, *run_e;
	GC_TRY(mem.alloc(&new_bw, pool->total_buckets));
	GC_TRY(mem.alloc(&keys, max_n));
	GC_TRY(mem.alloc(&keys_out, max_n));
	GC_TRY(mem.alloc(&vals, max_n));
	GC_TRY(mem.alloc(&vals_out, max_n));
	GC_TRY(mem.alloc(&run_b, max_nb));
	GC_TRY(mem.alloc(&run_e, max_nb));
	size_t sort_bytes = 0;
	GC_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, keys, keys_out, vals, vals_out, (int)std::max<uint64_t>(max_n, 1),
	                                        0, 32, st));
	unsigned char *sort_tmp;
	GC_TRY(mem.alloc(&sort_tmp, sort_bytes));
	std::vector<u32 *> lvl_words(L, nullptr), lvl_lens(L, nullptr);
	for (uint32_t l = L; l-- > 0;) {
		const uint32_t n = g[l + 1] - g[l];
		const bool leaf = l == L - 1;
		GC_TRY(mem.alloc(&lvl_words[l], (uint64_t)n * (leaf ? 2 : 9)));
		if (leaf) {
			k_gc_leaf_layout<<<grid_for(1ull << cfg.bucket_bits_each_level[l], sms), kGcBlock, 0, st>>>(
			    P, bm, prefix, G, g[l], newp, lvl_words[l], new_bw, err);
			continue;
		}
		GC_TRY(mem.alloc(&lvl_lens[l], n));
		const uint32_t bits = cfg.bucket_bits_each_level[l];
		GC_CUDA(cudaMemsetAsync(run_b, 0, (1ull << bits) * 4, st));
		GC_CUDA(cudaMemsetAsync(run_e, 0, (1ull << bits) * 4, st));
		if (n) {
			k_gc_inner_prep<<<grid_for(n, sms), kGcBlock, 0, st>>>(P, bm, prefix, G, g[l], n, l, newp, lvl_words[l],
			                                                       lvl_lens[l], keys, vals);
			const u32 *sorted_keys = keys, *sorted_vals = vals;
			if (bits) { // stable: equal keys keep rank order
				GC_CUDA(cub::DeviceRadixSort::SortPairs(sort_tmp, sort_bytes, keys, keys_out, vals, vals_out, (int)n, 0,
				                                        (int)bits, st));
				sorted_keys = keys_out;
				sorted_vals = vals_out;
			}
			k_gc_runs<<<grid_for(n, sms), kGcBlock, 0, st>>>(sorted_keys, n, run_b, run_e);
			k_gc_inner_layout<<<grid_for(1ull << bits, sms), kGcBlock, 0, st>>>(P, l, run_b, run_e, sorted_vals,
			                                                                    lvl_lens[l], g[l], newp, new_bw, err);
		} else {
			k_gc_inner_layout<<<grid_for(1ull << bits, sms), kGcBlock, 0, st>>>(P, l, run_b, run_e, vals, lvl_lens[l],
			                                                                    g[l], newp, new_bw, err);
		}
		GC_CUDA(cudaGetLastError());
	}
	GC_CUDA(cudaGetLastError());

	// 5. pages
	u32 *pages, *page_base;
	GC_TRY(mem.alloc(&pages, pool->total_buckets + 1));
	GC_TRY(mem.alloc(&page_base, pool->total_buckets + 1));
	GC_CUDA(cudaMemsetAsync(pages + pool->total_buckets, 0, 4, st));
	k_gc_page_counts<<<grid_for(pool->total_buckets, sms), kGcBlock, 0, st>>>(new_bw, (u32)pool->total_buckets,
	                                                                          cfg.word_bits_per_page, pages);
	size_t scan2 = 0;
	GC_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan2, pages, page_base, (int)(pool->total_buckets + 1), st));
	unsigned char *scan_tmp;
	GC_TRY(mem.alloc(&scan_tmp, scan2));
	GC_CUDA(cub::DeviceScan::ExclusiveSum(scan_tmp, scan2, pages, page_base, (int)(pool->total_buckets + 1), st));
	uint32_t used_pages = 0;
	GC_CUDA(cudaMemcpyAsync(&used_pages, page_base + pool->total_buckets, 4, cudaMemcpyDeviceToHost, st));
	GC_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, st));
	GC_CUDA(cudaStreamSynchronize(st));
	if (h_err & kGcErrBucket) {
		fprintf(stderr, "hashdag_gb300: hd_gc: a bucket cannot hold the nodes that hash to it after compaction\n");
		return HD_ERR_BUCKET_FULL;
	}
	if (!P.identity && (uint64_t)used_pages + 1 > P.heap_pages)
		return HD_ERR_POOL_OOM;
	if (stats) {
		std::vector<uint32_t> bw_old(pool->total_buckets);
		GC_CUDA(cudaMemcpyAsync(bw_old.data(), P.bucket_words, pool->total_buckets * 4, cudaMemcpyDeviceToHost, st));
		uint32_t heap_next = 0;
		GC_CUDA(cudaMemcpyAsync(&heap_next, P.counters + kCtrHeapNext, 4, cudaMemcpyDeviceToHost, st));
		GC_CUDA(cudaStreamSynchronize(st));
		uint64_t words_before = 0;
		for (uint32_t v : bw_old)
			words_before += v;
		stats->live_nodes = live;
		stats->words_before = words_before;
		stats->pages_before = std::min<uint64_t>(heap_next, P.heap_pages) - 1;
		stats->pages_after = used_pages;
	}

	// 6. write: nothing above changed the pool; from here on it is rewritten
	GC_CUDA(cudaMemsetAsync(P.page_table, 0xFF, pool->total_pages * 4, st));
	k_gc_page_table<<<grid_for(pool->total_buckets, sms), kGcBlock, 0, st>>>(P, (u32)pool->total_buckets, pages,
	                                                                         page_base);
	const uint64_t wp = 1ull << cfg.word_bits_per_page;
	if (P.identity)
		GC_CUDA(cudaMemsetAsync(P.heap, 0, (uint64_t)P.heap_pages * wp * 4, st));
	else
		GC_CUDA(cudaMemsetAsync(P.heap + wp, 0, (uint64_t)used_pages * wp * 4, st));
	for (uint32_t l = 0; l < L; ++l) {
		const uint32_t n = g[l + 1] - g[l];
		if (n)
			k_gc_write<<<grid_for(n, sms), kGcBlock, 0, st>>>(P, newp, g[l], n, lvl_words[l], lvl_lens[l],
			                                                  l == L - 1 ? 2u : 9u);
	}
	GC_CUDA(cudaMemcpyAsync(P.bucket_words, new_bw, pool->total_buckets * 4, cudaMemcpyDeviceToDevice, st));
	const uint32_t heap_next = used_pages + 1u;
	GC_CUDA(cudaMemcpyAsync(P.counters + kCtrHeapNext, &heap_next, 4, cudaMemcpyHostToDevice, st));
	if (n_roots) {
		GC_CUDA(cudaMemcpyAsync(d_roots, roots, n_roots * 4, cudaMemcpyHostToDevice, st));
		k_gc_remap_roots<<<grid_for(n_roots, sms), kGcBlock, 0, st>>>(bm, prefix, newp, d_roots, n_roots);
		GC_CUDA(cudaMemcpyAsync(roots, d_roots, n_roots * 4, cudaMemcpyDeviceToHost, st));
	}
	GC_CUDA(cudaGetLastError());
	GC_CUDA(cudaStreamSynchronize(st));
	pool->has_checkpoint = false; // its index and page table describe the old layout
	GC_TRY(hd_rebuild_index(pool, st));
	GC_TRY(hd_remake_filled(pool));
	if (stats) {
		std::vector<uint32_t> bw_new(pool->total_buckets);
		GC_CUDA(cudaMemcpyAsync(bw_new.data(), P.bucket_words, pool->total_buckets * 4, cudaMemcpyDeviceToHost, st));
		GC_CUDA(cudaStreamSynchronize(st));
		uint64_t words_after = 0;
		for (uint32_t v : bw_new)
			words_after += v;
		stats->words_after = words_after;
	}
	return HD_OK;
}

} // namespace

extern "C" hd_status hd_gc(hd_pool *pool, uint32_t *roots, uint32_t n_roots, hd_gc_stats *stats) {
	if (!pool || (n_roots && !roots))
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	if (cudaSetDevice(pool->device) != cudaSuccess)
		return HD_ERR_CUDA;
	if (cudaEventSynchronize(pool->ws_free) != cudaSuccess) // the pool's last pass or upsert has finished
		return HD_ERR_CUDA;
	if (stats)
		*stats = hd_gc_stats{};
	cudaStream_t st = nullptr;
	if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
		return HD_ERR_CUDA;
	++pool->epoch; // even a failed collection is treated as a rewrite (mirrors re-read everything)
	hd_status s = gc_impl(pool, roots, n_roots, stats, st);
	cudaStreamSynchronize(st);
	cudaStreamDestroy(st);
	return s;
}
