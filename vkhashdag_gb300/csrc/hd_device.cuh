// hd_device.cuh -- device-side building blocks of the HashDAG edit engine:
// pool view, node addressing, hashes, editor predicates, the dedup index
// encoding and the edit workspace layout.  Included by every .cu file.
#pragma once

#include "../../include/hashdag_gpu.h"

#include <cstdint>
#include <cuda_runtime.h>

namespace hd {

using u32 = uint32_t;
using u64 = uint64_t;

static constexpr u32 kNull = 0xFFFFFFFFu;
static constexpr u32 kMaxNodeLevels = 21; // node coordinates packed 21 bits per axis
static constexpr u32 kUnallocPage = 0xFFFFFFFFu;
static constexpr u32 kZeroPage = 0u; // physical page 0 is never handed out (failed allocations map here)

// device error codes (sticky, first error wins)
enum DevError : u32 {
	kErrNone = 0,
	kErrBucketFull = HD_ERR_BUCKET_FULL,
	kErrOom = HD_ERR_POOL_OOM,
	kErrIndexFull = HD_ERR_INDEX_FULL,
	kErrCapacity = HD_ERR_CAPACITY,
	kErrTimeout = HD_ERR_TIMEOUT,
	kErrInvalidRoot = HD_ERR_INVALID_ARG,
	kErrInternal = HD_ERR_INTERNAL,
};

// Config<uint32_t> with the derived per-level tables (include/hashdag/Config.hpp:15-57)
// and the filled node of every level (include/hashdag/NodePool.hpp:54).
struct DevConfig {
	u32 wbpp, pbpb, L, hasher;
	u32 bucket_bits[HD_MAX_LEVELS];
	u32 bucket_base[HD_MAX_LEVELS];
	u32 filled[HD_MAX_LEVELS];
};

// Device-resident node pool.  Pointers are the reference's virtual word
// indices; page_table maps a virtual page (bucket << pbpb | slot) to a
// physical page of the heap.
struct DevPool {
	DevConfig cfg;
	u32 *bucket_words; // [total_buckets]
	u32 *page_table;   // [total_pages] physical page or kUnallocPage
	u32 *heap;         // [heap_pages << wbpp]
	u32 *counters;     // [0] next physical page, [1] sticky error, [2] index slots used
	unsigned long long *index; // dedup index [index_mask+1]
	u64 index_mask;
	u64 total_pages;
	u32 heap_pages;
	u32 identity; // 1: the heap spans every virtual page, page i is physical page i
};

enum CounterSlot : u32 { kCtrHeapNext = 0, kCtrError = 1, kCtrIndexUsed = 2, kCtrCount = 4 };

__device__ __forceinline__ u32 wpp(const DevConfig &c) { return 1u << c.wbpp; }

// NodePool.hpp:75-77 read_node: one load with an identity-mapped heap, else
// through the page table.
__device__ __forceinline__ const u32 *node_addr(const DevPool &p, u32 ptr) {
	if (p.identity)
		return p.heap + ptr;
	u32 phys = __ldg(p.page_table + (ptr >> p.cfg.wbpp));
	return p.heap + ((u64)phys << p.cfg.wbpp) + (ptr & (wpp(p.cfg) - 1u));
}
// A page whose allocation failed maps to the zero page (paged heaps only).
__device__ __forceinline__ bool page_lost(const DevPool &p, u32 phys) { return !p.identity && phys == kZeroPage; }

__device__ __forceinline__ void set_error(u32 *slot, u32 code) { atomicCAS(slot, 0u, code); }

// ------------------------------------------------------------------ hashes
// include/hashdag/Hasher.hpp:21-39: MurmurHash3 x86-32 body, seed 0, length = words
struct Murmur {
	u32 h = 0;
	__host__ __device__ __forceinline__ void add(u32 k) {
		k *= 0xcc9e2d51u;
		k = (k << 15) | (k >> 17);
		k *= 0x1b873593u;
		h ^= k;
		h = (h << 13) | (h >> 19);
		h = h * 5u + 0xe6546b64u;
	}
	__host__ __device__ __forceinline__ u32 finish(u32 n) const {
		u32 x = h ^ n;
		x ^= x >> 16;
		x *= 0x85ebca6bu;
		x ^= x >> 13;
		x *= 0xc2b2ae35u;
		x ^= x >> 16;
		return x;
	}
};
// include/hashdag/Hasher.hpp:40-48: 64-bit finaliser truncated to 32 bits (leaves)
__host__ __device__ __forceinline__ u32 hash_leaf(u64 v) {
	v ^= v >> 33;
	v *= 0xff51afd7ed558ccdull;
	v ^= v >> 33;
	v *= 0xc4ceb9fe1a85ec53ull;
	v ^= v >> 33;
	return (u32)v;
}

__device__ __forceinline__ u64 mix64(u64 x) {
	x ^= x >> 30;
	x *= 0xbf58476d1ce4e5b9ull;
	x ^= x >> 27;
	x *= 0x94d049bb133111ebull;
	x ^= x >> 31;
	return x;
}

// ------------------------------------------------------------------ dedup index
// 64-bit slots of an open-addressing table over all nodes of the pool:
//   empty      ~0
//   committed  tag31 << 32 | node pointer           (bit 63 clear)
//   pending    1 << 63 | tag31 << 32 | item index    (claimed in this pass, not yet written)
//   tombstone  1 << 63 | 0x7FFFFFFF << 32 | 0xFFFFFFFE (claim of a failed insert)
// tag31 = low 31 bits of the node's content hash.
static constexpr unsigned long long kSlotEmpty = ~0ull;
static constexpr unsigned long long kSlotTomb = (1ull << 63) | (0x7FFFFFFFull << 32) | 0xFFFFFFFEull;
__device__ __forceinline__ u64 index_start(u32 h, u32 level, u64 mask) {
	return mix64(((u64)h << 8) | level) & mask;
}

// ------------------------------------------------------------------ editors
// src/main.cpp:32-150 (stateless forms).  Classification of a node at `level`
// with integer position pos[] against one edit: 0 kNotAffected, 1 kProceed,
// 2 full cover (kFill for FILL, kClear for DIG).
enum Cls : u32 { kClsNone = 0, kClsPartial = 1, kClsFull = 2 };

__host__ __device__ __forceinline__ u32 classify(const hd_edit_desc &e, u32 shift, u32 px, u32 py, u32 pz) {
	u32 lb[3] = {px << shift, py << shift, pz << shift};
	u32 ub[3] = {(px + 1u) << shift, (py + 1u) << shift, (pz + 1u) << shift};
	if (e.shape == HD_SHAPE_AABB) { // AABBEditor::EditNode (src/main.cpp:36-47)
		bool out = false, in = true;
#pragma unroll
		for (int a = 0; a < 3; ++a) {
			out |= (ub[a] <= e.p0[a]) | (lb[a] >= e.p1[a]);
			in &= (lb[a] >= e.p0[a]) & (ub[a] <= e.p1[a]);
		}
		return out ? kClsNone : (in ? kClsFull : kClsPartial);
	}
	// SphereEditor::EditNode (src/main.cpp:77-106), same integer formulas.
	// When every bound and the centre are <= 2^15, each distance is within
	// +-2^15, each square <= 2^30 and each sum of three < 2^32, so 32-bit
	// arithmetic is exact; clamping r2 to 2^32-1 keeps both comparisons exact.
	if (((ub[0] | ub[1] | ub[2]) <= 0x8000u) && ((e.p0[0] | e.p0[1] | e.p0[2]) < 0x8000u)) {
		const u32 r2c = e.r2 > 0xFFFFFFFFull ? 0xFFFFFFFFu : (u32)e.r2;
		u32 mx32 = 0, mn32 = 0;
#pragma unroll
		for (int a = 0; a < 3; ++a) {
			const int lbd = (int)lb[a] - (int)e.p0[a], ubd = (int)ub[a] - (int)e.p0[a];
			const u32 l2 = (u32)(lbd * lbd), u2 = (u32)(ubd * ubd);
			mx32 += l2 > u2 ? l2 : u2;
			mn32 += (lbd > 0 ? l2 : 0u) + (ubd < 0 ? u2 : 0u);
		}
		if (mx32 <= r2c)
			return kClsFull;
		return mn32 > r2c ? kClsNone : kClsPartial;
	}
	u64 mx = 0, mn = 0;
#pragma unroll
	for (int a = 0; a < 3; ++a) {
		long long lbd = (long long)lb[a] - (long long)e.p0[a];
		long long ubd = (long long)ub[a] - (long long)e.p0[a];
		u64 l2 = (u64)lbd * (u64)lbd, u2 = (u64)ubd * (u64)ubd;
		mx += l2 > u2 ? l2 : u2;
		mn += (lbd > 0 ? l2 : 0ull) + (ubd < 0 ? u2 : 0ull);
	}
	if (mx <= e.r2)
		return kClsFull;
	return mn > e.r2 ? kClsNone : kClsPartial;
}

// Classification of the 8 children (cells of 2^shift voxels) of the node at
// coordinate (px, py, pz) against one edit, 2 bits per child c (x half c&1,
// y half c>>1&1, z half c>>2&1): kClsNone / kClsPartial / kClsFull.  The
// formulas of classify() (AABBEditor / SphereEditor::EditNode,
// src/main.cpp:36-47,77-106) with each axis's terms of the node's two halves
// computed once for the 4 children sharing them.
template <typename I, typename U>
__host__ __device__ __forceinline__ u32 classify_children_sphere(const hd_edit_desc &e, const u32 o[3], u32 sz, U r2) {
	U mx[3][2], mn[3][2];
#pragma unroll
	for (int a = 0; a < 3; ++a) {
		const I d0 = (I)o[a] - (I)e.p0[a], d1 = d0 + (I)sz, d2 = d1 + (I)sz;
		const U s0 = (U)d0 * (U)d0, s1 = (U)d1 * (U)d1, s2 = (U)d2 * (U)d2;
		mx[a][0] = s0 > s1 ? s0 : s1;
		mx[a][1] = s1 > s2 ? s1 : s2;
		mn[a][0] = (d0 > 0 ? s0 : (U)0) + (d1 < 0 ? s1 : (U)0);
		mn[a][1] = (d1 > 0 ? s1 : (U)0) + (d2 < 0 ? s2 : (U)0);
	}
	u32 r = 0;
#pragma unroll
	for (u32 c = 0; c < 8; ++c) {
		const u32 hx = c & 1u, hy = (c >> 1) & 1u, hz = (c >> 2) & 1u;
		const U M = mx[0][hx] + mx[1][hy] + mx[2][hz], N = mn[0][hx] + mn[1][hy] + mn[2][hz];
		r |= (M <= r2 ? kClsFull : (N > r2 ? kClsNone : kClsPartial)) << (2u * c);
	}
	return r;
}
__host__ __device__ __forceinline__ u32 classify_children(const hd_edit_desc &e, u32 shift, u32 px, u32 py, u32 pz) {
	const u32 sz = 1u << shift;
	const u32 o[3] = {px << (shift + 1u), py << (shift + 1u), pz << (shift + 1u)};
	if (e.shape == HD_SHAPE_AABB) {
		u32 out[3], in[3]; // bit h: half h of the axis
#pragma unroll
		for (int a = 0; a < 3; ++a) {
			out[a] = in[a] = 0;
#pragma unroll
			for (u32 h = 0; h < 2; ++h) {
				const u32 lb = o[a] + sz * h, ub = lb + sz;
				out[a] |= ((ub <= e.p0[a]) | (lb >= e.p1[a])) ? 1u << h : 0u;
				in[a] |= ((lb >= e.p0[a]) & (ub <= e.p1[a])) ? 1u << h : 0u;
			}
		}
		u32 r = 0;
#pragma unroll
		for (u32 c = 0; c < 8; ++c) {
			const u32 hx = c & 1u, hy = (c >> 1) & 1u, hz = (c >> 2) & 1u;
			const bool o_ = ((out[0] >> hx) | (out[1] >> hy) | (out[2] >> hz)) & 1u;
			const bool i_ = ((in[0] >> hx) & (in[1] >> hy) & (in[2] >> hz)) & 1u;
			r |= (o_ ? kClsNone : (i_ ? kClsFull : kClsPartial)) << (2u * c);
		}
		return r;
	}
	// exact in 32 bits when every bound and the centre are <= 2^15 (as in classify)
	if (o[0] + 2u * sz <= 0x8000u && o[1] + 2u * sz <= 0x8000u && o[2] + 2u * sz <= 0x8000u &&
	    (e.p0[0] | e.p0[1] | e.p0[2]) < 0x8000u)
		return classify_children_sphere<int, u32>(e, o, sz, e.r2 > 0xFFFFFFFFull ? 0xFFFFFFFFu : (u32)e.r2);
	return classify_children_sphere<long long, u64>(e, o, sz, (u64)e.r2);
}

// Leaf voxel index i in [0,64) -> offset inside the 4^3 leaf (NodeCoord.hpp:32-43):
//   x = (i>>2 & 2) | (i & 1), y = (i>>3 & 2) | (i>>1 & 1), z = (i>>4 & 2) | (i>>2 & 1)
// 64-bit mask of the leaf voxels at origin (ox,oy,oz) inside the edit's shape
// (SphereEditor/AABBEditor::VoxelInRange, src/main.cpp:55-57,121-126).
// Sphere mask in 64-bit arithmetic (r2 > 2^30); rare, kept out of line.
static __host__ __device__ __noinline__ u64 sphere_mask_wide(const hd_edit_desc &e, u32 ox, u32 oy, u32 oz) {
	u64 dx2[4], dy2[4], dz2[4];
#pragma unroll
	for (u32 k = 0; k < 4; ++k) {
		const long long dx = (long long)(ox + k) - (long long)e.p0[0];
		const long long dy = (long long)(oy + k) - (long long)e.p0[1];
		const long long dz = (long long)(oz + k) - (long long)e.p0[2];
		dx2[k] = (u64)dx * (u64)dx;
		dy2[k] = (u64)dy * (u64)dy;
		dz2[k] = (u64)dz * (u64)dz;
	}
	u64 m = 0;
	for (u32 yo = 0; yo < 4; ++yo)
		for (u32 zo = 0; zo < 4; ++zo) {
			const u64 t = dy2[yo] + dz2[zo];
			const u32 base = ((yo & 1u) << 1) | ((zo & 1u) << 2) | ((yo >> 1) << 4) | ((zo >> 1) << 5);
			if (t > e.r2)
				continue;
			const u64 rem = e.r2 - t;
			const u32 nib = u32(dx2[0] <= rem) | u32(dx2[1] <= rem) << 1 | u32(dx2[2] <= rem) << 8 | u32(dx2[3] <= rem) << 9;
			m |= (u64)nib << base;
		}
	return m;
}

// 4-bit mask of the offsets k in 0..3 with lo <= o + k < hi.
__host__ __device__ __forceinline__ u32 axis_run(u32 o, u32 lo, u32 hi) {
	const u32 a = lo > o ? (lo - o < 4u ? lo - o : 4u) : 0u, b = hi > o ? (hi - o < 4u ? hi - o : 4u) : 0u;
	return b > a ? ((1u << b) - 1u) & ~((1u << a) - 1u) : 0u;
}
// The leaf's voxels whose offset along one axis is in m (bit k: offset k), in
// the voxel order above: the pattern of that axis's 4 offsets (index bits 0,3
// for x, 1,4 for y, 2,5 for z) copied over the other index bits by one
// multiply; the copies land on disjoint bits, so nothing carries.
__host__ __device__ __forceinline__ u64 spread_x(u32 m) { return (u64)((m & 3u) | ((m & 0xCu) << 6)) * 0x0055005500550055ull; }
__host__ __device__ __forceinline__ u64 spread_y(u32 m) {
	return (u64)((m & 1u) | ((m & 2u) << 1) | ((m & 4u) << 14) | ((m & 8u) << 15)) * 0x0000333300003333ull;
}
__host__ __device__ __forceinline__ u64 spread_z(u32 m) {
	return ((u64)((m & 1u) | ((m & 2u) << 3)) | ((u64)(m & 4u) << 30) | ((u64)(m & 8u) << 33)) * 0x0F0F0F0Full;
}

// acc shifted left by one with the sign bit of t appended (a funnel shift).
__host__ __device__ __forceinline__ u32 push_sign(u32 acc, u32 t) {
#ifdef __CUDA_ARCH__
	return __funnelshift_l(t, acc, 1);
#else
	return (acc << 1) | (t >> 31);
#endif
}

__host__ __device__ __forceinline__ u64 shape_mask(const hd_edit_desc &e, u32 ox, u32 oy, u32 oz) {
	// The leaf's voxels are 16 x-rows of 4 (one per (y,z) offset pair).  Row
	// (yo,zo) holds voxel indices base+{0,1,8,9} for x offsets 0..3, with
	// base = (yo&1)<<1 | (zo&1)<<2 | (yo>>1)<<4 | (zo>>1)<<5.
	if (e.shape == HD_SHAPE_AABB) { // separable: the voxels whose x, y and z offsets are all inside
		return spread_x(axis_run(ox, e.p0[0], e.p1[0])) & spread_y(axis_run(oy, e.p0[1], e.p1[1])) &
		       spread_z(axis_run(oz, e.p0[2], e.p1[2]));
	}
	// A leaf that the sphere only partially covers lies within r+4 of the centre
	// on every axis, so for r2 <= 2^30 every square and every sum of three fits
	// in 32 bits (3 * 32772^2 < 2^32); the wider form handles the rest.
	if (e.r2 <= (1ull << 29)) {
		// Here every square is below 2^29 + 2^18 and a voxel's
		// t = dx^2 + dy^2 + dz^2 - r2 - 1 lies in (-2^30, 2^31): it is negative
		// exactly when the voxel is inside, so its sign bit is the voxel's bit.
		// One three-input add per voxel, and the sign bits shifted into each
		// half of the mask in voxel order (index 63 first).
		u32 sx[4], sy[4], sz[4];
		const int cx = (int)e.p0[0], cy = (int)e.p0[1], cz = (int)e.p0[2];
		const u32 r2m = (u32)e.r2 + 1u;
#pragma unroll
		for (u32 k = 0; k < 4; ++k) {
			const int dx = (int)(ox + k) - cx, dy = (int)(oy + k) - cy, dz = (int)(oz + k) - cz;
			sx[k] = (u32)(dx * dx);
			sy[k] = (u32)(dy * dy);
			sz[k] = (u32)(dz * dz) - r2m;
		}
		u32 hi = 0, lo = 0;
#pragma unroll
		for (int i = 63; i >= 32; --i)
			hi = push_sign(hi, sx[((i >> 2) & 2) | (i & 1)] + sy[((i >> 3) & 2) | ((i >> 1) & 1)] + sz[((i >> 4) & 2) | ((i >> 2) & 1)]);
#pragma unroll
		for (int i = 31; i >= 0; --i)
			lo = push_sign(lo, sx[((i >> 2) & 2) | (i & 1)] + sy[((i >> 3) & 2) | ((i >> 1) & 1)] + sz[((i >> 4) & 2) | ((i >> 2) & 1)]);
		return (u64)lo | ((u64)hi << 32);
	}
	if (e.r2 <= (1ull << 30)) {
		u32 dx2[4], dy2[4], dz2[4];
		const int cx = (int)e.p0[0], cy = (int)e.p0[1], cz = (int)e.p0[2];
#pragma unroll
		for (u32 k = 0; k < 4; ++k) {
			const int dx = (int)(ox + k) - cx, dy = (int)(oy + k) - cy, dz = (int)(oz + k) - cz;
			dx2[k] = (u32)(dx * dx);
			dy2[k] = (u32)(dy * dy);
			dz2[k] = (u32)(dz * dz);
		}
		const u32 r2 = (u32)e.r2;
		// voxel in iff dx2 + dy2 <= r2 - dz2 (for a z slab with dz2 <= r2); every
		// dx2 + dy2 < 2^32 since each square is < 2^30 + 2^18 + 16
		u32 xy[4][4];
#pragma unroll
		for (u32 yo = 0; yo < 4; ++yo)
#pragma unroll
			for (u32 k = 0; k < 4; ++k)
				xy[yo][k] = dx2[k] + dy2[yo];
		u32 lo = 0, hi = 0;
#pragma unroll
		for (u32 zo = 0; zo < 4; ++zo) {
			const bool okz = dz2[zo] <= r2;
			const u32 rz = r2 - dz2[zo];
#pragma unroll
			for (u32 yo = 0; yo < 4; ++yo) {
				u32 nib = u32(xy[yo][0] <= rz) | u32(xy[yo][1] <= rz) << 1 | u32(xy[yo][2] <= rz) << 8 |
				          u32(xy[yo][3] <= rz) << 9;
				nib = okz ? nib : 0u;
				const u32 base = ((yo & 1u) << 1) | ((zo & 1u) << 2) | ((yo >> 1) << 4) | ((zo >> 1) << 5);
				if (base < 32u)
					lo |= nib << base;
				else
					hi |= nib << (base - 32u);
			}
		}
		return (u64)lo | ((u64)hi << 32);
	}
	return sphere_mask_wide(e, ox, oy, oz);
}

// One voxel inside the edit's shape (VoxelInRange, src/main.cpp:55-57,121-126).
__host__ __device__ __forceinline__ bool voxel_in(const hd_edit_desc &e, u32 x, u32 y, u32 z) {
	if (e.shape == HD_SHAPE_AABB)
		return x >= e.p0[0] && y >= e.p0[1] && z >= e.p0[2] && x < e.p1[0] && y < e.p1[1] && z < e.p1[2];
	const long long dx = (long long)x - (long long)e.p0[0], dy = (long long)y - (long long)e.p0[1],
	                dz = (long long)z - (long long)e.p0[2];
	return (u64)dx * (u64)dx + (u64)dy * (u64)dy + (u64)dz * (u64)dz <= e.r2;
}

__device__ __forceinline__ u64 pack_pos(u32 x, u32 y, u32 z) { return (u64)x | ((u64)y << 21) | ((u64)z << 42); }
__device__ __forceinline__ u32 pos_x(u64 p) { return (u32)(p & 0x1FFFFFu); }
__device__ __forceinline__ u32 pos_y(u64 p) { return (u32)((p >> 21) & 0x1FFFFFu); }
__device__ __forceinline__ u32 pos_z(u64 p) { return (u32)((p >> 42) & 0x1FFFFFu); }

// ------------------------------------------------------------------ edit workspace
// Frontier items of one batched edit pass.  Inner items (levels 0..L-2) live
// in one index space, every level a contiguous range in level order.  The
// leaf level has no items: the kernel of level L-2 computes the 8 child leaves
// of each node itself and emits only the changed leaves as candidates
// (Workspace::leaf, with their bits in leaf_new).
struct Items {
	u64 *pos;     // packed node coordinate (inner items)
	u32 *base;    // node the edit list applies to (original node, filled node or Null) (inner items)
	u32 *parent;  // child slot of the parent (inner index*8 + child) or kNull for the root
	u32 *lst_off; // edit list [lst_off, lst_off+lst_len) in Workspace::lists (inner items)
	u32 *lst_len;
	u32 *res;     // result pointer of items without a parent (the root item, upsert calls)
	u64 cap;
};

struct Workspace {
	Items inner, leaf; // leaf: candidates (parent slot, res)
	u32 *bchild;       // [inner.cap*8] children of the base node
	u32 *cnew;         // [inner.cap*8] new children
	u64 *leaf_new;     // [leaf.cap] bits of the leaf candidates
	u32 *lists;        // edit lists
	u64 list_cap;
	u32 *long_q;       // per inner level: items with long edit lists (same index space as inner)
	u32 *todo;         // [inner.cap] level-(L-2) items that still need the claiming probe
	u32 *todo_parent;  // [inner.cap] their parents' child slots (todo record t: bchild/cnew slot begin(L-2)+t)
	u32 *leaf_cls;     // [inner.cap] one-edit level-(L-2) items: their 8 leaves' classes | fill << 16 (leaf_classes)
	// Leaf-pattern cache of the leaf kernels: leaf bits -> pointer of the
	// resident leaf with those bits, 2-way sets of slots (2k, 2k+1), a slot
	// 16 bytes (key, then the pointer's complement), cleared to zero at the
	// start of every multi-kernel pass (key 0 = empty, stored 0 = pointer not
	// yet written).  A pass's changed leaves repeat few patterns (a box
	// face cuts every leaf it crosses the same way), so most of its read-only
	// leaf lookups are answered from this L2-resident table instead of a
	// random index slot and a random heap read.  lc_key null: not used.
	unsigned long long *lc_key; // [2 * (lc_mask + 1)]: per slot the key, then ~pointer
	u32 lc_mask;
	const hd_edit_desc *edits;
	u32 n_edits;
	u32 long_threshold; // lists longer than this are expanded by a block (inner) or a warp (level L-2)
	// non-null for passes replayed from a CUDA graph: [0] = number of edits,
	// [1] = input root, written before each replay (the graph's kernels keep
	// the parameters they were captured with)
	const u32 *pass_desc;
	// device counters (u64 so that overflow counts stay exact):
	//   [0..L-1)     items per inner level, [L-1] leaf candidates
	//   [32..)       long items per level
	//   [64]         list entries used
	//   [65]         workspace error
	//   [66]         root result, [67] input root
	//   [96..96+L)   candidates per level, [128..) words of candidates,
	//   [160..) inserted per level, [192..) words inserted
	unsigned long long *ctr;
};

enum WsCtr : u32 {
	kWsItems = 0,
	kWsLong = 32,
	kWsList = 64,
	kWsError = 65,
	kWsRoot = 66,
	kWsRootIn = 67,
	kWsMaxProbe = 68,   // longest index probe of the pass
	kWsProbeSteps = 69, // index slots visited in the pass
	kWsCasRetry = 70,   // failed bucket-count CAS attempts
	kWsTodo = 71,       // entries in Workspace::todo
	// work of the level-(L-2) leaf kernels (the algorithmic bytes of that phase)
	kWsLeafNodes = 72,   // level-(L-2) nodes rebuilt
	kWsLeafPairs = 73,   // (node, edit) pairs: edit-list entries of those nodes
	kWsLeafBaseW = 74,   // words of their base nodes read
	kWsLeafOld = 75,     // old leaves read from the heap
	kWsLeafLookup = 76,  // read-only lookups of changed leaves
	kWsLeafCacheHit = 77, // of these, answered by the leaf-pattern cache
	kWsLeafInner = 78,    // read-only index lookups of level-(L-2) nodes whose children are all known
	kWsCand = 96,
	kWsCandWords = 128,
	kWsIns = 160,
	kWsInsWords = 192,
	kWsCtrCount = 224,
};

} // namespace hd
