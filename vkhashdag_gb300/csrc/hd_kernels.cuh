// hd_kernels.cuh -- kernels of the level-synchronous HashDAG edit pass.
//
// One pass applies an ordered list of edits to a root and rebuilds the
// touched subtrees bottom-up, like NodePoolBase::edit_node / edit_leaf
// (include/hashdag/NodePool.hpp:319-396) applied edit after edit, but with
// every level of every edit processed by one set of launches:
//
//   k_root            classify the root against the whole edit list
//   k_expand_short(l) thread per level-l node: classify its 8 children against
//                     the node's edit list, keep the edits after the last full
//                     cover (EditType kFill/kClear), emit children to recurse
//   k_expand_long(l)  same, a warp per node, for nodes with long edit lists
//   k_leaf            thread per leaf: apply the leaf's edit list to its 64 voxels
//   k_probe(l)        build each level-l node, hash it (Hasher.hpp:21-48) and
//                     find-or-claim it in the dedup index; claimed nodes
//                     reserve words in their bucket (page padding rule of
//                     NodePool.hpp:134-157) and open pages from the heap
//   k_commit(l)       write claimed nodes, publish them in the index, hand
//                     every node's pointer to its parent's child slot
//   k_finish          report the root
//
// Per voxel the result equals applying the edits one after another: the last
// edit whose shape covers the voxel decides, and a node is replaced by the
// filled node / Null only when the last covering edit covers all of it.
#pragma once

#include "hd_device.cuh"

namespace hd {

static constexpr u32 kFullMask = 0xFFFFFFFFu;
static constexpr int kBlock = 256;

__device__ __forceinline__ u32 lane_id() { return threadIdx.x & 31u; }

// Exclusive offset of this lane's `count` within a warp-wide reservation on *ctr.
// All 32 lanes must call it.
__device__ __forceinline__ u64 warp_reserve(unsigned long long *ctr, u32 count) {
	u32 lane = lane_id();
	u32 incl = count;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		u32 v = __shfl_up_sync(kFullMask, incl, d);
		if (lane >= (u32)d)
			incl += v;
	}
	u32 total = __shfl_sync(kFullMask, incl, 31);
	unsigned long long base = 0;
	if (lane == 31 && total)
		base = atomicAdd(ctr, (unsigned long long)total);
	base = __shfl_sync(kFullMask, base, 31);
	return base + incl - count;
}

// Level ranges: inner levels 0..L-2 share the inner index space in level order,
// the leaf level starts at 0 of the leaf space.
__device__ __forceinline__ void level_range(const Workspace &W, u32 L, u32 l, u64 &begin, u64 &n) {
	if (l == L - 1) {
		begin = 0;
		n = W.ctr[kWsItems + l];
		if (n > W.leaf.cap)
			n = W.leaf.cap;
		return;
	}
	u64 b = 0;
	for (u32 k = 0; k < l; ++k)
		b += W.ctr[kWsItems + k];
	begin = b;
	n = W.ctr[kWsItems + l];
	if (begin >= W.inner.cap)
		n = 0;
	else if (begin + n > W.inner.cap)
		n = W.inner.cap - begin;
}
// First index of level l in its space (used when emitting level l items).
__device__ __forceinline__ u64 level_begin(const Workspace &W, u32 L, u32 l) {
	if (l == L - 1)
		return 0;
	u64 b = 0;
	for (u32 k = 0; k < l; ++k)
		b += W.ctr[kWsItems + k];
	return b;
}

__device__ __forceinline__ bool ws_failed(const Workspace &W) { return *(volatile unsigned long long *)&W.ctr[kWsError] != 0; }
__device__ __forceinline__ bool pool_failed(const DevPool &P) { return *(volatile u32 *)&P.counters[kCtrError] != 0; }

// Children of a base node (NodePool.hpp:278-309 get_unpacked_node_array; the
// filled node's children are the filled node of the level below).
__device__ __forceinline__ void base_children(const DevPool &P, u32 l, u32 b, u32 out[8]) {
	if (b == kNull) {
#pragma unroll
		for (int c = 0; c < 8; ++c)
			out[c] = kNull;
		return;
	}
	if (b == P.cfg.filled[l]) {
		u32 f = P.cfg.filled[l + 1];
#pragma unroll
		for (int c = 0; c < 8; ++c)
			out[c] = f;
		return;
	}
	const u32 *p = node_addr(P, b);
	u32 mask = p[0] & 0xFFu;
	u32 k = 1;
#pragma unroll
	for (int c = 0; c < 8; ++c) {
		if ((mask >> c) & 1u)
			out[c] = p[k++];
		else
			out[c] = kNull;
	}
}

// Whether an edit that only partially covers a node can change it, given the
// node's base: a dig cannot change an empty node and a fill cannot change a
// full one.  Leading edits that cannot change the node are dropped.
__device__ __forceinline__ bool effective(u32 op, u32 base, u32 filled) {
	if (base == kNull)
		return op == HD_OP_FILL;
	if (base == filled)
		return op == HD_OP_DIG;
	return true;
}

template <bool Identity>
__device__ __forceinline__ u32 list_at(const Workspace &W, u32 off, u32 p) {
	return Identity ? p : W.lists[off + p];
}

// Plan of one child against the parent's edit list, by one thread.
// Returns the number of edits to keep (0 = terminal, result in *base_out).
template <bool Identity>
__device__ __forceinline__ u32 plan_child_thread(const Workspace &W, u32 off, u32 len, u32 shift, u32 cx, u32 cy,
                                                 u32 cz, u32 old, u32 filled, u32 *base_out, u32 *first_out) {
	int lastfull = -1;
	u32 lastop = 0;
	for (u32 p = 0; p < len; ++p) {
		const hd_edit_desc &e = W.edits[list_at<Identity>(W, off, p)];
		if (classify(e, shift, cx, cy, cz) == kClsFull) {
			lastfull = (int)p;
			lastop = e.op;
		}
	}
	u32 base = lastfull >= 0 ? (lastop == HD_OP_FILL ? filled : kNull) : old;
	*base_out = base;
	u32 first = kNull, cnt = 0;
	for (u32 p = (u32)(lastfull + 1); p < len; ++p) {
		const hd_edit_desc &e = W.edits[list_at<Identity>(W, off, p)];
		if (classify(e, shift, cx, cy, cz) == kClsPartial) {
			if (first == kNull && effective(e.op, base, filled))
				first = p;
			if (first != kNull)
				++cnt;
		}
	}
	*first_out = first;
	return cnt;
}

// Writes the kept edits of a planned child (positions >= first, partial) in order.
template <bool Identity>
__device__ __forceinline__ void write_child_list_thread(const Workspace &W, u32 off, u32 len, u32 first, u32 shift,
                                                        u32 cx, u32 cy, u32 cz, u32 *dst) {
	u32 k = 0;
	for (u32 p = first; p < len; ++p) {
		u32 id = list_at<Identity>(W, off, p);
		if (classify(W.edits[id], shift, cx, cy, cz) == kClsPartial)
			dst[k++] = id;
	}
}

struct ChildSpace {
	Items *it;
	u64 begin;
	u64 cap;
};

__device__ __forceinline__ Items &items_of(Workspace &W, u32 L, u32 l) { return l == L - 1 ? W.leaf : W.inner; }

// ------------------------------------------------------------------ k_expand_short
// Thread per level-l inner node with an edit list of at most long_threshold edits.
__global__ void __launch_bounds__(kBlock) k_expand_short(DevPool P, Workspace W, u32 l) {
	if (ws_failed(W)) // an earlier launch overflowed: some items were never written
		return;
	const u32 L = P.cfg.L;
	const u32 cl = l + 1;
	u64 begin, n;
	level_range(W, L, l, begin, n);
	const u64 child_begin = level_begin(W, L, cl);
	Items &child = items_of(W, L, cl);
	const u32 shift = P.cfg.L + 1u - cl; // child bounds at voxel level
	const u32 filled_c = P.cfg.filled[cl];
	const u64 stride = (u64)gridDim.x * blockDim.x;
	for (u64 w0 = (u64)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
		const u64 t = w0 + lane_id();
		const bool valid = t < n;
		const u64 i = begin + t;
		u32 len = 0, off = 0, b = kNull;
		u64 pos = 0;
		if (valid) {
			len = W.inner.lst_len[i];
			off = W.inner.lst_off[i];
			b = W.inner.base[i];
			pos = W.inner.pos[i];
		}
		const bool mine = valid && len <= W.long_threshold;
		u32 cbase[8], cfirst[8], ccnt[8];
		u32 n_emit = 0, n_list = 0, n_long = 0;
		u32 old[8];
		if (mine) {
			base_children(P, l, b, old);
			const u32 px = pos_x(pos), py = pos_y(pos), pz = pos_z(pos);
#pragma unroll 1
			for (u32 c = 0; c < 8; ++c) {
				const u32 cx = (px << 1) | (c & 1u), cy = (py << 1) | ((c >> 1) & 1u), cz = (pz << 1) | ((c >> 2) & 1u);
				ccnt[c] = plan_child_thread<false>(W, off, len, shift, cx, cy, cz, old[c], filled_c, &cbase[c], &cfirst[c]);
				if (ccnt[c]) {
					++n_emit;
					n_list += ccnt[c];
					n_long += (cl < L - 1 && ccnt[c] > W.long_threshold) ? 1u : 0u;
				}
			}
		}
		const u64 item0 = warp_reserve(&W.ctr[kWsItems + cl], n_emit);
		const u64 list0 = warp_reserve(&W.ctr[kWsList], n_list);
		const u64 long0 = (cl < L - 1) ? warp_reserve(&W.ctr[kWsLong + cl], n_long) : 0;
		if (!mine)
			continue;
		u32 res[8];
		u64 it = child_begin + item0, lo = list0, lg = long0;
		const u32 px = pos_x(pos), py = pos_y(pos), pz = pos_z(pos);
#pragma unroll 1
		for (u32 c = 0; c < 8; ++c) {
			if (!ccnt[c]) {
				res[c] = cbase[c];
				continue;
			}
			res[c] = kNull; // overwritten by the child's commit
			const u32 cx = (px << 1) | (c & 1u), cy = (py << 1) | ((c >> 1) & 1u), cz = (pz << 1) | ((c >> 2) & 1u);
			if (it < child.cap && lo + ccnt[c] <= W.list_cap) {
				child.pos[it] = pack_pos(cx, cy, cz);
				child.base[it] = cbase[c];
				child.parent[it] = (u32)(i * 8u + c);
				child.lst_off[it] = (u32)lo;
				child.lst_len[it] = ccnt[c];
				write_child_list_thread<false>(W, off, len, cfirst[c], shift, cx, cy, cz, W.lists + lo);
				if (cl < L - 1 && ccnt[c] > W.long_threshold) {
					if (child_begin + lg < W.inner.cap)
						W.long_q[child_begin + lg] = (u32)it;
					else
						atomicCAS(&W.ctr[kWsError], 0ull, (unsigned long long)kErrCapacity);
					++lg;
				}
			} else {
				atomicCAS(&W.ctr[kWsError], 0ull, (unsigned long long)kErrCapacity);
			}
			++it;
			lo += ccnt[c];
		}
		uint4 *bc = reinterpret_cast<uint4 *>(W.bchild + i * 8u);
		uint4 *cn = reinterpret_cast<uint4 *>(W.cnew + i * 8u);
		bc[0] = make_uint4(old[0], old[1], old[2], old[3]);
		bc[1] = make_uint4(old[4], old[5], old[6], old[7]);
		cn[0] = make_uint4(res[0], res[1], res[2], res[3]);
		cn[1] = make_uint4(res[4], res[5], res[6], res[7]);
	}
}

// ------------------------------------------------------------------ warp planning (long lists)
// Plan of one child by a whole warp: returns kept-count upper bound, base and first.
template <bool Identity>
__device__ __forceinline__ u32 plan_child_warp(const Workspace &W, u32 off, u32 len, u32 shift, u32 cx, u32 cy, u32 cz,
                                               u32 old, u32 filled, u32 *base_out, u32 *first_out) {
	const u32 lane = lane_id();
	u32 lf1 = 0; // lastfull + 1
	for (u32 p = lane; p < len; p += 32) {
		const hd_edit_desc &e = W.edits[list_at<Identity>(W, off, p)];
		if (classify(e, shift, cx, cy, cz) == kClsFull)
			lf1 = p + 1;
	}
	lf1 = __reduce_max_sync(kFullMask, lf1);
	u32 base = old;
	if (lf1)
		base = W.edits[list_at<Identity>(W, off, lf1 - 1)].op == HD_OP_FILL ? filled : kNull;
	u32 first = kNull, cnt = 0;
	for (u32 p = lf1 + lane; p < len; p += 32) {
		const hd_edit_desc &e = W.edits[list_at<Identity>(W, off, p)];
		if (classify(e, shift, cx, cy, cz) == kClsPartial) {
			++cnt;
			if (first == kNull && effective(e.op, base, filled))
				first = p;
		}
	}
	first = __reduce_min_sync(kFullMask, first);
	cnt = __reduce_add_sync(kFullMask, cnt);
	*base_out = base;
	*first_out = first;
	return first == kNull ? 0u : cnt; // cnt bounds the kept edits (positions >= first)
}

// Writes kept edits (positions >= first, partial) in order; returns the count.
template <bool Identity>
__device__ __forceinline__ u32 write_child_list_warp(const Workspace &W, u32 off, u32 len, u32 first, u32 shift, u32 cx,
                                                     u32 cy, u32 cz, u32 *dst) {
	const u32 lane = lane_id();
	u32 k = 0;
	for (u32 p0 = first; p0 < len; p0 += 32) {
		const u32 p = p0 + lane;
		u32 id = 0;
		bool keep = false;
		if (p < len) {
			id = list_at<Identity>(W, off, p);
			keep = classify(W.edits[id], shift, cx, cy, cz) == kClsPartial;
		}
		const u32 bal = __ballot_sync(kFullMask, keep);
		if (keep)
			dst[k + __popc(bal & ((1u << lane) - 1u))] = id;
		k += __popc(bal);
	}
	return k;
}

// Emits one child planned by a warp; lane 0 reserves.  The list gets the
// upper bound `cnt` of entries and the exact kept count is stored as its length.
template <bool Identity>
__device__ __forceinline__ void emit_child_warp(Workspace &W, u32 L, u32 cl, u64 child_begin, u32 parent_slot, u32 off,
                                                u32 len, u32 shift, u32 cx, u32 cy, u32 cz, u32 base, u32 first, u32 cnt) {
	Items &child = items_of(W, L, cl);
	unsigned long long it = 0, lo = 0;
	if (lane_id() == 0) {
		it = atomicAdd(&W.ctr[kWsItems + cl], 1ull);
		lo = atomicAdd(&W.ctr[kWsList], (unsigned long long)cnt);
	}
	it = __shfl_sync(kFullMask, it, 0) + child_begin;
	lo = __shfl_sync(kFullMask, lo, 0);
	if (it < child.cap && lo + cnt <= W.list_cap) {
		const u32 k = write_child_list_warp<Identity>(W, off, len, first, shift, cx, cy, cz, W.lists + lo);
		if (lane_id() == 0) {
			child.pos[it] = pack_pos(cx, cy, cz);
			child.base[it] = base;
			child.parent[it] = parent_slot;
			child.lst_off[it] = (u32)lo;
			child.lst_len[it] = k;
			if (cl < L - 1 && k > W.long_threshold) {
				const unsigned long long lg = atomicAdd(&W.ctr[kWsLong + cl], 1ull);
				if (child_begin + lg < W.inner.cap)
					W.long_q[child_begin + lg] = (u32)it;
				else
					atomicCAS(&W.ctr[kWsError], 0ull, (unsigned long long)kErrCapacity);
			}
		}
	} else if (lane_id() == 0) {
		atomicCAS(&W.ctr[kWsError], 0ull, (unsigned long long)kErrCapacity);
	}
}

// ------------------------------------------------------------------ k_expand_long
// Warp per level-l node whose edit list is longer than long_threshold.
__global__ void __launch_bounds__(kBlock) k_expand_long(DevPool P, Workspace W, u32 l) {
	if (ws_failed(W))
		return;
	const u32 L = P.cfg.L;
	const u32 cl = l + 1;
	const u64 begin = level_begin(W, L, l);
	u64 n = W.ctr[kWsLong + l];
	const u64 child_begin = level_begin(W, L, cl);
	const u32 shift = P.cfg.L + 1u - cl;
	const u32 filled_c = P.cfg.filled[cl];
	const u64 warps = (u64)gridDim.x * (blockDim.x / 32);
	for (u64 q = (u64)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; q < n; q += warps) {
		const u64 qi = begin + q;
		if (qi >= W.inner.cap)
			break;
		const u64 i = W.long_q[qi];
		const u32 len = W.inner.lst_len[i], off = W.inner.lst_off[i], b = W.inner.base[i];
		const u64 pos = W.inner.pos[i];
		u32 old[8], res[8];
		base_children(P, l, b, old);
		const u32 px = pos_x(pos), py = pos_y(pos), pz = pos_z(pos);
		for (u32 c = 0; c < 8; ++c) {
			const u32 cx = (px << 1) | (c & 1u), cy = (py << 1) | ((c >> 1) & 1u), cz = (pz << 1) | ((c >> 2) & 1u);
			u32 cb, cf;
			u32 cnt = plan_child_warp<false>(W, off, len, shift, cx, cy, cz, old[c], filled_c, &cb, &cf);
			if (!cnt) {
				res[c] = cb;
				continue;
			}
			res[c] = kNull;
			emit_child_warp<false>(W, L, cl, child_begin, (u32)(i * 8u + c), off, len, shift, cx, cy, cz, cb, cf, cnt);
		}
		if (lane_id() == 0) {
			uint4 *bc = reinterpret_cast<uint4 *>(W.bchild + i * 8u);
			uint4 *cn = reinterpret_cast<uint4 *>(W.cnew + i * 8u);
			bc[0] = make_uint4(old[0], old[1], old[2], old[3]);
			bc[1] = make_uint4(old[4], old[5], old[6], old[7]);
			cn[0] = make_uint4(res[0], res[1], res[2], res[3]);
			cn[1] = make_uint4(res[4], res[5], res[6], res[7]);
		}
	}
}

// ------------------------------------------------------------------ k_root
// One warp: NodePool.hpp:405-414 edit_switch on the root for the whole list.
__global__ void k_root(DevPool P, Workspace W, u32 root_val, const u32 *root_ptr) {
	if (threadIdx.x >= 32)
		return;
	const u32 L = P.cfg.L;
	const u32 root = root_ptr ? *root_ptr : root_val;
	if (lane_id() == 0)
		W.ctr[kWsRootIn] = root;
	// a root must be Null or point into a page that holds data
	if (root != kNull) {
		const u64 vp = root >> P.cfg.wbpp;
		const u32 phys = vp < P.total_pages ? P.page_table[vp] : kUnallocPage;
		if (phys == kUnallocPage || phys == kZeroPage) {
			if (lane_id() == 0) {
				W.ctr[kWsRoot] = root;
				atomicCAS(&W.ctr[kWsError], 0ull, (unsigned long long)kErrInvalidRoot);
			}
			return;
		}
	}
	u32 b, f;
	u32 cnt = plan_child_warp<true>(W, 0, W.n_edits, L + 1u, 0, 0, 0, root, P.cfg.filled[0], &b, &f);
	if (!cnt) {
		if (lane_id() == 0)
			W.ctr[kWsRoot] = b;
		return;
	}
	emit_child_warp<true>(W, L, 0, 0, kNull, 0, W.n_edits, L + 1u, 0, 0, 0, b, f, cnt);
}

// ------------------------------------------------------------------ k_leaf
// Thread per leaf: NodePool.hpp:319-343 for the leaf's edit list, 64 voxels at a time.
__global__ void __launch_bounds__(kBlock) k_leaf(DevPool P, Workspace W) {
	if (ws_failed(W))
		return;
	const u32 L = P.cfg.L;
	u64 begin, n;
	level_range(W, L, L - 1, begin, n);
	const u32 filled = P.cfg.filled[L - 1];
	const u64 stride = (u64)gridDim.x * blockDim.x;
	for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
		const u64 i = begin + t;
		const u32 b = W.leaf.base[i];
		u64 bits0 = 0;
		if (b == filled)
			bits0 = ~0ull;
		else if (b != kNull) {
			const u32 *p = node_addr(P, b);
			bits0 = (u64)p[0] | ((u64)p[1] << 32);
		}
		const u64 pos = W.leaf.pos[i];
		const u32 ox = pos_x(pos) << 2, oy = pos_y(pos) << 2, oz = pos_z(pos) << 2;
		const u32 off = W.leaf.lst_off[i], len = W.leaf.lst_len[i];
		u64 bits = bits0;
		for (u32 p = 0; p < len; ++p) {
			const hd_edit_desc &e = W.edits[W.lists[off + p]];
			const u64 m = shape_mask(e, ox, oy, oz);
			bits = e.op == HD_OP_FILL ? (bits | m) : (bits & ~m);
		}
		W.leaf_new[i] = bits;
		W.leaf.state[i] = bits == bits0 ? kStUnchanged : (bits == 0 ? kStEmpty : kStCand);
	}
}

// ------------------------------------------------------------------ dedup: find or claim
struct NodeWords {
	u32 w[9];
	u32 n;
};

__device__ __forceinline__ bool equal_resident(const DevPool &P, u32 ptr, const NodeWords &nw) {
	const u32 *p = node_addr(P, ptr);
	for (u32 k = 0; k < nw.n; ++k)
		if (p[k] != nw.w[k])
			return false;
	return true;
}

// Reserve space for a node of w words in bucket b (NodePool.hpp:134-157 on an
// atomic word count).  Returns false when the bucket is full.
__device__ __forceinline__ bool reserve(const DevPool &P, u32 b, u32 w, u32 *ptr_out, u32 *pad_out) {
	const u32 wp = wpp(P.cfg), wpb = 1u << (P.cfg.wbpp + P.cfg.pbpb);
	u32 old = *(volatile u32 *)&P.bucket_words[b];
	u32 off, nw;
	for (;;) {
		off = old;
		if ((off & (wp - 1u)) + w > wp)
			off = (off | (wp - 1u)) + 1u;
		nw = off + w;
		if (nw > wpb)
			return false;
		u32 prev = atomicCAS(&P.bucket_words[b], old, nw);
		if (prev == old)
			break;
		old = prev;
	}
	*pad_out = off != old ? old : kNull;
	const u32 vpage = (b << P.cfg.pbpb) | (off >> P.cfg.wbpp);
	if ((off & (wp - 1u)) == 0u) {
		u32 phys = atomicAdd(&P.counters[kCtrHeapNext], 1u);
		if (phys >= P.heap_pages) {
			phys = kZeroPage;
			set_error(&P.counters[kCtrError], kErrOom);
		}
		P.page_table[vpage] = phys;
	}
	*ptr_out = (b << (P.cfg.wbpp + P.cfg.pbpb)) | off;
	return true;
}

// Find-or-claim of one candidate.  Compare(j) tests equality with pending item j.
template <typename CmpPending>
__device__ __forceinline__ void find_or_claim(const DevPool &P, Items &it, u64 i, u32 level, u32 h, u32 bucket,
                                              const NodeWords &nw, CmpPending &&cmp_pending) {
	const u64 mask = P.index_mask;
	const unsigned long long tag = (unsigned long long)(h & 0x7FFFFFFFu) << 32;
	const u32 bucket_shift = P.cfg.wbpp + P.cfg.pbpb;
	u64 s = index_start(h, level, mask);
	for (u64 probe = 0; probe <= mask; ++probe, s = (s + 1) & mask) {
		unsigned long long v = *(volatile unsigned long long *)&P.index[s];
		if (v == kSlotEmpty) {
			const unsigned long long claim = (1ull << 63) | tag | (unsigned long long)i;
			unsigned long long prev = atomicCAS(&P.index[s], kSlotEmpty, claim);
			if (prev == kSlotEmpty) {
				u32 ptr, pad;
				if (reserve(P, bucket, nw.n, &ptr, &pad)) {
					it.state[i] = kStRep;
					it.res[i] = ptr;
					it.pad[i] = pad;
				} else {
					set_error(&P.counters[kCtrError], kErrBucketFull);
					it.state[i] = kStFail;
					it.res[i] = kNull;
				}
				it.link[i] = (u32)s; // index slot
				return;
			}
			v = prev;
		}
		if (v == kSlotTomb || ((v >> 32) & 0x7FFFFFFFull) != (tag >> 32))
			continue;
		const u32 val = (u32)v;
		if (v >> 63) { // pending in this pass
			if (cmp_pending(val)) {
				it.state[i] = kStAlias;
				it.link[i] = val;
				return;
			}
		} else if ((val >> bucket_shift) == bucket && equal_resident(P, val, nw)) {
			it.state[i] = kStFound;
			it.res[i] = val;
			return;
		}
	}
	set_error(&P.counters[kCtrError], kErrIndexFull);
	it.state[i] = kStFail;
	it.res[i] = kNull;
	it.link[i] = kNull;
}

__device__ __forceinline__ void warp_count(unsigned long long *ctr, u32 v) {
	v = __reduce_add_sync(kFullMask, v);
	if (lane_id() == 0 && v)
		atomicAdd(ctr, (unsigned long long)v);
}

// ------------------------------------------------------------------ k_probe
template <bool Leaf>
__global__ void __launch_bounds__(kBlock) k_probe(DevPool P, Workspace W, u32 l) {
	if (ws_failed(W))
		return;
	__shared__ int s_skip;
	if (threadIdx.x == 0)
		s_skip = pool_failed(P) ? 1 : 0;
	__syncthreads();
	const bool skip = s_skip != 0;
	const u32 L = P.cfg.L;
	u64 begin, n;
	level_range(W, L, l, begin, n);
	Items &it = Leaf ? W.leaf : W.inner;
	const u32 nb_mask = (1u << P.cfg.bucket_bits[l]) - 1u;
	const u32 bbase = P.cfg.bucket_base[l];
	const bool zero_hash = P.cfg.hasher == HD_HASHER_ZERO;
	const u64 stride = (u64)gridDim.x * blockDim.x;
	for (u64 w0 = (u64)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
		const u64 t = w0 + lane_id();
		u32 cand = 0, cwords = 0;
		if (t < n) {
			const u64 i = begin + t;
			NodeWords nw;
			u32 h;
			if (skip) { // an earlier level failed: insert nothing more
				if (!Leaf || it.state[i] == kStCand) {
					it.state[i] = kStFail;
					it.link[i] = kNull;
				}
				goto next;
			}
			if (Leaf) {
				if (it.state[i] != kStCand)
					goto next;
				const u64 bits = W.leaf_new[i];
				nw.w[0] = (u32)bits;
				nw.w[1] = (u32)(bits >> 32);
				nw.n = 2;
				h = hash_leaf(bits);
			} else {
				const uint4 *cn4 = reinterpret_cast<const uint4 *>(W.cnew + i * 8u);
				const uint4 *bc4 = reinterpret_cast<const uint4 *>(W.bchild + i * 8u);
				const uint4 a0 = cn4[0], a1 = cn4[1], b0 = bc4[0], b1 = bc4[1];
				const u32 c[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
				if (a0.x == b0.x && a0.y == b0.y && a0.z == b0.z && a0.w == b0.w && a1.x == b1.x && a1.y == b1.y &&
				    a1.z == b1.z && a1.w == b1.w) {
					it.state[i] = kStUnchanged;
					goto next;
				}
				u32 mask = 0, k = 1;
				Murmur mm;
#pragma unroll
				for (int q = 0; q < 8; ++q)
					if (c[q] != kNull) {
						mask |= 1u << q;
						nw.w[k++] = c[q];
					}
				if (!mask) {
					it.state[i] = kStEmpty;
					goto next;
				}
				nw.w[0] = mask;
				nw.n = k;
				for (u32 q = 0; q < k; ++q)
					mm.add(nw.w[q]);
				h = mm.finish(k);
			}
			{
				const u32 bucket = bbase + ((zero_hash ? 0u : h) & nb_mask);
				cand = 1;
				cwords = nw.n;
				if (Leaf) {
					const u64 mine = W.leaf_new[i];
					find_or_claim(P, it, i, l, h, bucket, nw, [&](u32 j) { return W.leaf_new[j] == mine; });
				} else {
					const uint4 *cn4 = reinterpret_cast<const uint4 *>(W.cnew + i * 8u);
					const uint4 a0 = cn4[0], a1 = cn4[1];
					find_or_claim(P, it, i, l, h, bucket, nw, [&](u32 j) {
						const uint4 *o4 = reinterpret_cast<const uint4 *>(W.cnew + (u64)j * 8u);
						const uint4 c0 = o4[0], c1 = o4[1];
						return c0.x == a0.x && c0.y == a0.y && c0.z == a0.z && c0.w == a0.w && c1.x == a1.x &&
						       c1.y == a1.y && c1.z == a1.z && c1.w == a1.w;
					});
				}
			}
		}
	next:
		warp_count(&W.ctr[kWsCand + l], cand);
		warp_count(&W.ctr[kWsCandWords + l], cwords);
	}
}

// ------------------------------------------------------------------ k_commit
template <bool Leaf>
__global__ void __launch_bounds__(kBlock) k_commit(DevPool P, Workspace W, u32 l) {
	if (ws_failed(W))
		return;
	const u32 L = P.cfg.L;
	u64 begin, n;
	level_range(W, L, l, begin, n);
	Items &it = Leaf ? W.leaf : W.inner;
	const u32 wp = wpp(P.cfg);
	const u32 bucket_shift = P.cfg.wbpp + P.cfg.pbpb;
	const u64 stride = (u64)gridDim.x * blockDim.x;
	for (u64 w0 = (u64)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
		const u64 t = w0 + lane_id();
		u32 ins = 0, insw = 0;
		if (t < n) {
			const u64 i = begin + t;
			const u32 st = it.state[i];
			u32 r;
			switch (st) {
			case kStUnchanged:
				r = it.base[i];
				break;
			case kStEmpty:
				r = kNull;
				break;
			case kStFound:
				r = it.res[i];
				break;
			case kStAlias:
				r = it.res[it.link[i]];
				break;
			case kStRep: {
				r = it.res[i];
				const u32 slot = it.link[i];
				const u32 phys = P.page_table[r >> P.cfg.wbpp];
				if (phys == kZeroPage) {
					P.index[slot] = kSlotTomb;
					r = kNull;
					break;
				}
				u32 *dst = P.heap + ((u64)phys << P.cfg.wbpp) + (r & (wp - 1u));
				if (Leaf) {
					const u64 bits = W.leaf_new[i];
					dst[0] = (u32)bits;
					dst[1] = (u32)(bits >> 32);
					insw = 2;
				} else {
					const uint4 *cn4 = reinterpret_cast<const uint4 *>(W.cnew + i * 8u);
					const uint4 a0 = cn4[0], a1 = cn4[1];
					const u32 c[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
					u32 mask = 0, k = 1;
#pragma unroll
					for (int q = 0; q < 8; ++q)
						if (c[q] != kNull) {
							mask |= 1u << q;
							dst[k++] = c[q];
						}
					dst[0] = mask;
					insw = k;
				}
				const u32 pad = it.pad[i];
				if (pad != kNull) {
					const u32 vp = ((r >> bucket_shift) << P.cfg.pbpb) | (pad >> P.cfg.wbpp);
					const u32 zp = P.page_table[vp];
					if (zp != kUnallocPage && zp != kZeroPage) {
						u32 *z = P.heap + ((u64)zp << P.cfg.wbpp);
						for (u32 q = pad & (wp - 1u); q < wp; ++q)
							z[q] = 0u;
					}
				}
				ins = 1;
				__threadfence();
				const unsigned long long pend = P.index[slot];
				P.index[slot] = (((pend >> 32) & 0x7FFFFFFFull) << 32) | r;
				break;
			}
			default: // kStFail
				if (it.link[i] != kNull)
					P.index[it.link[i]] = kSlotTomb;
				r = kNull;
				break;
			}
			it.res[i] = r;
			const u32 ps = it.parent[i];
			if (ps == kNull)
				W.ctr[kWsRoot] = r;
			else
				W.cnew[ps] = r;
		}
		warp_count(&W.ctr[kWsIns + l], ins);
		warp_count(&W.ctr[kWsInsWords + l], insw);
	}
}

// ------------------------------------------------------------------ k_finish
__global__ void k_finish(DevPool P, Workspace W, u32 *out_root) {
	if (threadIdx.x != 0)
		return;
	u64 ins = 0;
	for (u32 l = 0; l < P.cfg.L; ++l)
		ins += W.ctr[kWsIns + l];
	atomicAdd(&P.counters[kCtrIndexUsed], (u32)ins);
	const bool bad = W.ctr[kWsError] != 0 || P.counters[kCtrError] != 0;
	const u32 r = bad ? (u32)W.ctr[kWsRootIn] : (u32)W.ctr[kWsRoot];
	W.ctr[kWsRoot] = r;
	if (out_root)
		*out_root = r;
}

} // namespace hd
