// hd_kernels.cuh -- kernels of the level-synchronous HashDAG edit pass.
//
// One pass applies an ordered list of edits to a root and rebuilds the
// touched subtrees bottom-up, like NodePoolBase::edit_node / edit_leaf
// (include/hashdag/NodePool.hpp:319-396) applied edit after edit, but with
// every level of every edit processed by one set of launches:
//
//   k_root            classify the root against the whole edit list (one block)
//   k_expand_short(l) thread per level-l node (l <= L-3): classify its 8
//                     children against the node's edit list, keep the edits
//                     after the last full cover (EditType kFill/kClear), emit
//                     the children that still need work as level-(l+1) items
//   k_expand_long(l)  the same for nodes with long edit lists, a block per
//                     (node, child) with an order-preserving block compaction
//   k_leafparent      thread per level-(L-2) node (warp for long lists): apply
//                     the node's edit list to the 64 voxels of each of its 8
//                     child leaves (NodePool.hpp:319-343) and emit the changed
//                     leaves as dedup candidates
//   k_dedup(l)        hash each candidate (Hasher.hpp:21-48), merge equal
//                     candidates of a warp (__match_any_sync), find or insert
//                     it through the dedup index: a claimed node reserves
//                     words in its bucket (page padding rule of
//                     NodePool.hpp:134-157), opens pages from the heap, is
//                     written and published; every node's pointer goes to its
//                     parent's child slot
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
static constexpr int kLongBlock = 256;

__device__ __forceinline__ u32 lane_id() { return threadIdx.x & 31u; }

// Kernels replayed from a CUDA graph read the pass's edit count from device memory.
__device__ __forceinline__ void apply_pass_desc(Workspace &W) {
	if (W.pass_desc)
		W.n_edits = W.pass_desc[0];
}

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

// Level ranges: inner levels 0..L-2 share the inner index space in level order;
// the leaf candidates start at 0 of the leaf space.
__device__ __forceinline__ u64 level_begin(const Workspace &W, u32 L, u32 l) {
	if (l == L - 1)
		return 0;
	u64 b = 0;
	for (u32 k = 0; k < l; ++k)
		b += W.ctr[kWsItems + k];
	return b;
}
__device__ __forceinline__ void level_range(const Workspace &W, u32 L, u32 l, u64 &begin, u64 &n) {
	begin = level_begin(W, L, l);
	n = W.ctr[kWsItems + l];
	const u64 cap = l == L - 1 ? W.leaf.cap : W.inner.cap;
	if (begin >= cap)
		n = 0;
	else if (begin + n > cap)
		n = cap - begin;
}

__device__ __forceinline__ bool ws_failed(const Workspace &W) { return *(volatile unsigned long long *)&W.ctr[kWsError] != 0; }
__device__ __forceinline__ bool pool_failed(const DevPool &P) { return *(volatile u32 *)&P.counters[kCtrError] != 0; }
__device__ __forceinline__ void ws_error(Workspace &W, u32 code) { atomicCAS(&W.ctr[kWsError], 0ull, (unsigned long long)code); }

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

__device__ __forceinline__ u64 leaf_bits(const DevPool &P, u32 ptr) {
	if (ptr == kNull)
		return 0ull;
	if (ptr == P.cfg.filled[P.cfg.L - 1])
		return ~0ull;
	const u32 *p = node_addr(P, ptr);
	return (u64)p[0] | ((u64)p[1] << 32);
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

// Consistency check of an inner item's edit list before it is walked.
__device__ __forceinline__ bool list_ok(Workspace &W, u32 off, u32 len) {
	if (len > W.n_edits || (u64)off + len > W.list_cap) {
		ws_error(W, kErrInternal);
		return false;
	}
	return true;
}

template <bool Identity> __device__ __forceinline__ u32 list_at(const Workspace &W, u32 off, u32 p) {
	return Identity ? p : W.lists[off + p];
}

// An item with a single edit stores that edit's index in lst_off instead of
// the offset of a one-entry list: the kernel that expands it (or rebuilds its
// leaves) skips a dependent load, and the kernel that emits it writes one
// list entry less.  Every other item stores the offset of its list.  Lists
// longer than long_threshold (at least 1) are never direct.
__device__ __forceinline__ bool direct_edit(u32 len) { return len == 1u; }
// Edit p of an item's list.
__device__ __forceinline__ u32 item_list_at(const Workspace &W, u32 off, u32 len, u32 p) {
	return len == 1u ? off : W.lists[off + p];
}
// Consistency check of an item's edit list (or direct edit index).
__device__ __forceinline__ bool item_list_ok(Workspace &W, u32 off, u32 len) {
	if (len == 1u) {
		if (off >= W.n_edits) {
			ws_error(W, kErrInternal);
			return false;
		}
		return true;
	}
	return list_ok(W, off, len);
}

// The classes of a level-(L-2) node's 8 leaves under its one edit
// (classify_children at leaf size, 2 bits per leaf) and the edit's fill bit
// at bit 16: written by the kernel that emits the item, read by the
// compacted leaf kernel, which then needs neither the classification nor the
// edit record for the leaves it settles.
__device__ __forceinline__ u32 leaf_classes(const hd_edit_desc &e, u32 x, u32 y, u32 z) {
	return classify_children(e, 2u, x, y, z) | (e.op == HD_OP_FILL ? 1u << 16 : 0u);
}

__device__ __forceinline__ void child_pos(u64 pos, u32 c, u32 &cx, u32 &cy, u32 &cz) {
	cx = (pos_x(pos) << 1) | (c & 1u);
	cy = (pos_y(pos) << 1) | ((c >> 1) & 1u);
	cz = (pos_z(pos) << 1) | ((c >> 2) & 1u);
}

// ------------------------------------------------------------------ thread planning (short lists)
// Plan of one child against the parent's edit list, by one thread.
// Returns the number of edits to keep (0 = terminal, result in *base_out).
__device__ __forceinline__ u32 plan_child_thread(const Workspace &W, u32 off, u32 len, u32 shift, u32 cx, u32 cy,
                                                 u32 cz, u32 old, u32 filled, u32 *base_out, u32 *first_out) {
	int lastfull = -1;
	u32 lastop = 0;
	for (u32 p = 0; p < len; ++p) {
		const hd_edit_desc &e = W.edits[W.lists[off + p]];
		if (classify(e, shift, cx, cy, cz) == kClsFull) {
			lastfull = (int)p;
			lastop = e.op;
		}
	}
	const u32 base = lastfull >= 0 ? (lastop == HD_OP_FILL ? filled : kNull) : old;
	*base_out = base;
	u32 first = kNull, cnt = 0;
	for (u32 p = (u32)(lastfull + 1); p < len; ++p) {
		const hd_edit_desc &e = W.edits[W.lists[off + p]];
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
__device__ __forceinline__ void write_child_list_thread(const Workspace &W, u32 off, u32 len, u32 first, u32 shift,
                                                        u32 cx, u32 cy, u32 cz, u32 *dst) {
	u32 k = 0;
	for (u32 p = first; p < len; ++p) {
		const u32 id = W.lists[off + p];
		if (classify(W.edits[id], shift, cx, cy, cz) == kClsPartial)
			dst[k++] = id;
	}
}

// ------------------------------------------------------------------ k_expand_short
// Thread per level-l inner node (l <= L-3) with an edit list of at most
// long_threshold edits.  Children are inner items of level l+1.
//
// Staged form (k_expand_short): a warp's emitted children are written by all
// 32 lanes together instead of each node's lane walking its 8 child slots.
// The warp's children take consecutive item slots in lane order, so child q
// of the warp is item (warp base + q): every lane plans its node and stages
// what each of its children needs (base, edit count, kept edits, list
// offset) at that position in shared memory, then the lanes write the items
// 32 at a time (coalesced), with their edit lists, the long-list queue
// entries and, at level L-2, the leaf classes of one-edit items.
struct ExpandWarpStage {
	u64 pos[32];                       // the lane's node
	u32 item[32], off[32], len[32];    // its item index and edit list
	u32 base[256], cnt[256], keep[256], lo[256]; // per child of the warp, in item order
	unsigned char q[256];              // lane << 3 | child slot
};
template <bool Staged>
__device__ __forceinline__ void expand_short_phase(const DevPool &P, Workspace &W, u32 l, u64 tbase, u64 tstride,
                                                   ExpandWarpStage *S = nullptr) {
	if (ws_failed(W)) // an earlier launch overflowed: some items were never written
		return;
	const u32 L = P.cfg.L;
	const u32 cl = l + 1;
	u64 begin, n;
	level_range(W, L, l, begin, n);
	const u64 child_begin = level_begin(W, L, cl);
	const u32 shift = L + 1u - cl; // child bounds at voxel level
	const u32 filled_c = P.cfg.filled[cl];
	const u32 T = W.long_threshold;
	const u64 stride = tstride;
	for (u64 w0 = tbase + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
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
		const bool mine = valid && len <= T && item_list_ok(W, off, len);
		u32 cbase[8], cfirst[8], ccnt[8], old[8], part[8];
		u32 n_emit = 0, n_list = 0, n_long = 0;
		if (mine) {
			base_children(P, l, b, old);
			if (len <= 32u) {
				// one pass over the list: every edit read once and classified
				// against the 8 children together (bit p of full/part[c]: edit p
				// covers / partly covers child c; bit p of fills: edit p fills)
				u32 full[8], fills = 0;
#pragma unroll
				for (u32 c = 0; c < 8; ++c)
					full[c] = part[c] = 0;
				for (u32 p = 0; p < len; ++p) {
					const hd_edit_desc e = W.edits[item_list_at(W, off, len, p)];
					const u32 k = classify_children(e, shift, pos_x(pos), pos_y(pos), pos_z(pos));
					fills |= (e.op == HD_OP_FILL ? 1u : 0u) << p;
#pragma unroll
					for (u32 c = 0; c < 8; ++c) {
						const u32 kc = (k >> (2u * c)) & 3u;
						full[c] |= (kc == kClsFull ? 1u : 0u) << p;
						part[c] |= (kc == kClsPartial ? 1u : 0u) << p;
					}
				}
				// plan_child_thread from the bits: the last full cover sets the base;
				// the kept list starts at the first later partial edit that can change it
#pragma unroll
				for (u32 c = 0; c < 8; ++c) {
					const int lastfull = full[c] ? 31 - __clz(full[c]) : -1;
					const u32 base = lastfull >= 0 ? (((fills >> lastfull) & 1u) ? filled_c : kNull) : old[c];
					const u32 after = lastfull >= 0 ? (lastfull == 31 ? 0u : ~0u << (lastfull + 1)) : ~0u;
					const u32 eff = base == kNull ? fills : (base == filled_c ? ~fills : ~0u); // effective()
					const u32 cand = part[c] & after;
					const u32 f = cand & eff;
					cbase[c] = base;
					cfirst[c] = f ? (u32)(__ffs(f) - 1) : kNull;
					ccnt[c] = f ? (u32)__popc(cand & (~0u << cfirst[c])) : 0u;
					part[c] = cand & (f ? (~0u << cfirst[c]) : 0u); // the kept edits
					if (ccnt[c]) {
						++n_emit;
						n_list += direct_edit(ccnt[c]) ? 0u : ccnt[c];
						n_long += ccnt[c] > T ? 1u : 0u;
					}
				}
			} else {
#pragma unroll 1
				for (u32 c = 0; c < 8; ++c) {
					u32 cx, cy, cz;
					child_pos(pos, c, cx, cy, cz);
					ccnt[c] = plan_child_thread(W, off, len, shift, cx, cy, cz, old[c], filled_c, &cbase[c], &cfirst[c]);
					part[c] = 0;
					if (ccnt[c]) {
						++n_emit;
						n_list += direct_edit(ccnt[c]) ? 0u : ccnt[c];
						n_long += ccnt[c] > T ? 1u : 0u;
					}
				}
			}
		}
		const u64 item0 = warp_reserve(&W.ctr[kWsItems + cl], n_emit);
		const u64 list0 = warp_reserve(&W.ctr[kWsList], n_list);
		if (Staged) {
			const u32 lane = lane_id();
			const u64 wbase = __shfl_sync(kFullMask, item0, 0); // lane 0's slot opens the warp's range
			if (mine) {
				S->pos[lane] = pos;
				S->item[lane] = (u32)i;
				S->off[lane] = off;
				S->len[lane] = len;
				u32 q = (u32)(item0 - wbase);
				u64 lo = list0;
#pragma unroll 1
				for (u32 c = 0; c < 8; ++c) {
					if (!ccnt[c])
						continue;
					S->q[q] = (unsigned char)((lane << 3) | c);
					S->base[q] = cbase[c];
					S->cnt[q] = ccnt[c];
					S->keep[q] = len <= 32u ? part[c] : cfirst[c];
					S->lo[q] = lo < 0xFFFFFFFFull ? (u32)lo : 0xFFFFFFFFu; // past list_cap: fails the check below
					lo += direct_edit(ccnt[c]) ? 0u : ccnt[c];
					++q;
				}
				uint4 *bc = reinterpret_cast<uint4 *>(W.bchild + i * 8u);
				uint4 *cn = reinterpret_cast<uint4 *>(W.cnew + i * 8u);
				bc[0] = make_uint4(old[0], old[1], old[2], old[3]);
				bc[1] = make_uint4(old[4], old[5], old[6], old[7]);
				u32 res[8];
#pragma unroll
				for (u32 c = 0; c < 8; ++c)
					res[c] = ccnt[c] ? kNull : cbase[c]; // an emitted child's slot is written by its commit
				cn[0] = make_uint4(res[0], res[1], res[2], res[3]);
				cn[1] = make_uint4(res[4], res[5], res[6], res[7]);
			}
			const u32 total = __shfl_sync(kFullMask, (u32)(item0 - wbase) + n_emit, 31);
			__syncwarp();
			for (u32 j0 = 0; j0 < total; j0 += 32u) {
				const u32 j = j0 + lane;
				if (j >= total)
					continue;
				const u32 e = S->q[j], src = e >> 3, c = e & 7u;
				const u64 it = child_begin + wbase + j;
				const u32 cnt = S->cnt[j], slen = S->len[src], soff = S->off[src], kp = S->keep[j], lo = S->lo[j];
				const bool direct = direct_edit(cnt);
				const u32 n_entries = direct ? 0u : cnt;
				u32 cx, cy, cz;
				child_pos(S->pos[src], c, cx, cy, cz);
				if (it < W.inner.cap && (u64)lo + n_entries <= W.list_cap) {
					W.inner.pos[it] = pack_pos(cx, cy, cz);
					W.inner.base[it] = S->base[j];
					W.inner.parent[it] = S->item[src] * 8u + c;
					W.inner.lst_len[it] = cnt;
					if (direct) { // the one kept edit: the first set bit of keep / position keep
						const u32 id = slen <= 32u ? item_list_at(W, soff, slen, (u32)(__ffs(kp) - 1)) : W.lists[soff + kp];
						W.inner.lst_off[it] = id;
						if (cl + 2u == L)
							W.leaf_cls[it] = leaf_classes(W.edits[id], cx, cy, cz);
					} else {
						W.inner.lst_off[it] = lo;
						if (slen <= 32u) {
							u32 k = 0;
							for (u32 m = kp; m; m &= m - 1u)
								W.lists[lo + k++] = item_list_at(W, soff, slen, (u32)(__ffs(m) - 1));
						} else {
							write_child_list_thread(W, soff, slen, kp, shift, cx, cy, cz, W.lists + lo);
						}
					}
					if (cnt > T) { // rare: one queue slot each
						const unsigned long long lg = atomicAdd(&W.ctr[kWsLong + cl], 1ull);
						if (child_begin + lg < W.inner.cap)
							W.long_q[child_begin + lg] = (u32)it;
						else
							ws_error(W, kErrCapacity);
					}
				} else {
					ws_error(W, kErrCapacity);
				}
			}
			__syncwarp(); // the stage is rewritten by the next iteration
			continue;
		}
		const u64 long0 = warp_reserve(&W.ctr[kWsLong + cl], n_long);
		if (!mine)
			continue;
		u32 res[8];
		u64 it = child_begin + item0, lo = list0, lg = long0;
#pragma unroll 1
		for (u32 c = 0; c < 8; ++c) {
			if (!ccnt[c]) {
				res[c] = cbase[c];
				continue;
			}
			res[c] = kNull; // overwritten by the child's commit
			u32 cx, cy, cz;
			child_pos(pos, c, cx, cy, cz);
			const bool direct = direct_edit(ccnt[c]);
			const u32 n_entries = direct ? 0u : ccnt[c];
			if (it < W.inner.cap && lo + n_entries <= W.list_cap) {
				W.inner.pos[it] = pack_pos(cx, cy, cz);
				W.inner.base[it] = cbase[c];
				W.inner.parent[it] = (u32)(i * 8u + c);
				W.inner.lst_len[it] = ccnt[c];
				if (direct) { // the one kept edit: the first set bit of part / position cfirst
					const u32 id = len <= 32u ? item_list_at(W, off, len, (u32)(__ffs(part[c]) - 1)) : W.lists[off + cfirst[c]];
					W.inner.lst_off[it] = id;
					if (cl + 2u == L)
						W.leaf_cls[it] = leaf_classes(W.edits[id], cx, cy, cz);
				} else {
					W.inner.lst_off[it] = (u32)lo;
				}
				if (direct) {
				} else if (len <= 32u) {
					u32 k = 0;
					for (u32 m = part[c]; m; m &= m - 1u)
						W.lists[lo + k++] = item_list_at(W, off, len, (u32)(__ffs(m) - 1));
				} else {
					write_child_list_thread(W, off, len, cfirst[c], shift, cx, cy, cz, W.lists + lo);
				}
				if (ccnt[c] > T) {
					if (child_begin + lg < W.inner.cap)
						W.long_q[child_begin + lg] = (u32)it;
					else
						ws_error(W, kErrCapacity);
					++lg;
				}
			} else {
				ws_error(W, kErrCapacity);
			}
			++it;
			lo += n_entries;
		}
		uint4 *bc = reinterpret_cast<uint4 *>(W.bchild + i * 8u);
		uint4 *cn = reinterpret_cast<uint4 *>(W.cnew + i * 8u);
		bc[0] = make_uint4(old[0], old[1], old[2], old[3]);
		bc[1] = make_uint4(old[4], old[5], old[6], old[7]);
		cn[0] = make_uint4(res[0], res[1], res[2], res[3]);
		cn[1] = make_uint4(res[4], res[5], res[6], res[7]);
	}
}
// 4 blocks of 256 per SM (64 registers, a few spilled): 6.1 ms per step against 6.5 at 3 blocks
// (80 registers) and 7.2 at 2 (96) on the 32768^3 batch.
static __global__ void __launch_bounds__(kBlock, 4) k_expand_short(DevPool P, Workspace W, u32 l) {
	__shared__ ExpandWarpStage s_stage[kBlock / 32];
	apply_pass_desc(W);
	expand_short_phase<true>(P, W, l, (u64)blockIdx.x * blockDim.x, (u64)gridDim.x * blockDim.x,
	                         &s_stage[threadIdx.x >> 5]);
}

// ------------------------------------------------------------------ block planning (long lists)
// Block-wide reductions through a shared scratch of at least 33 words.
template <int Op> __device__ __forceinline__ u32 warp_red(u32 v) {
	return Op == 0 ? __reduce_max_sync(kFullMask, v) : (Op == 1 ? __reduce_min_sync(kFullMask, v) : __reduce_add_sync(kFullMask, v));
}
template <int Op> __device__ __forceinline__ u32 block_reduce(u32 v, u32 *sm) {
	const u32 warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	v = warp_red<Op>(v);
	if (lane_id() == 0)
		sm[warp] = v;
	__syncthreads();
	if (warp == 0) {
		u32 x = lane_id() < nw ? sm[lane_id()] : (Op == 1 ? kNull : 0u);
		x = warp_red<Op>(x);
		if (lane_id() == 0)
			sm[32] = x;
	}
	__syncthreads();
	const u32 r = sm[32];
	__syncthreads();
	return r;
}

// Plan of one child by a whole block: returns kept-count upper bound (0 = terminal).
template <bool Identity>
__device__ u32 plan_child_block(const Workspace &W, u32 off, u32 len, u32 shift, u32 cx, u32 cy, u32 cz, u32 old,
                                u32 filled, u32 *base_out, u32 *first_out, u32 *sm) {
	u32 lf1 = 0; // lastfull + 1
	for (u32 p = threadIdx.x; p < len; p += blockDim.x)
		if (classify(W.edits[list_at<Identity>(W, off, p)], shift, cx, cy, cz) == kClsFull)
			lf1 = p + 1;
	lf1 = block_reduce<0>(lf1, sm);
	u32 base = old;
	if (lf1)
		base = W.edits[list_at<Identity>(W, off, lf1 - 1)].op == HD_OP_FILL ? filled : kNull;
	u32 first = kNull, cnt = 0;
	for (u32 p = lf1 + threadIdx.x; p < len; p += blockDim.x) {
		const hd_edit_desc &e = W.edits[list_at<Identity>(W, off, p)];
		if (classify(e, shift, cx, cy, cz) == kClsPartial) {
			++cnt;
			if (first == kNull && effective(e.op, base, filled))
				first = p;
		}
	}
	first = block_reduce<1>(first, sm);
	cnt = block_reduce<2>(cnt, sm);
	*base_out = base;
	*first_out = first;
	return first == kNull ? 0u : cnt;
}

// Writes the kept edits (positions >= first, partial) in order; returns the count.
template <bool Identity>
__device__ u32 write_child_list_block(const Workspace &W, u32 off, u32 len, u32 first, u32 shift, u32 cx, u32 cy, u32 cz,
                                      u32 *dst, u32 *sm) {
	const u32 warp = threadIdx.x >> 5, nw = blockDim.x >> 5, lane = lane_id();
	u32 k = 0;
	for (u32 p0 = first; p0 < len; p0 += blockDim.x) {
		const u32 p = p0 + threadIdx.x;
		u32 id = 0;
		bool keep = false;
		if (p < len) {
			id = list_at<Identity>(W, off, p);
			keep = classify(W.edits[id], shift, cx, cy, cz) == kClsPartial;
		}
		const u32 bal = __ballot_sync(kFullMask, keep);
		if (lane == 0)
			sm[warp] = __popc(bal);
		__syncthreads();
		u32 before = 0, total = 0;
		for (u32 w = 0; w < nw; ++w) {
			const u32 c = sm[w];
			before += w < warp ? c : 0u;
			total += c;
		}
		if (keep)
			dst[k + before + __popc(bal & ((1u << lane) - 1u))] = id;
		k += total;
		__syncthreads();
	}
	return k;
}

// Emits one inner child item planned by a block; errors go to the workspace.
template <bool Identity>
__device__ void emit_child_block(Workspace &W, u32 L, u32 cl, u64 child_begin, u32 parent_slot, u32 off, u32 len,
                                 u32 shift, u32 cx, u32 cy, u32 cz, u32 base, u32 first, u32 cnt, u32 *sm) {
	if (threadIdx.x == 0) {
		sm[34] = (u32)atomicAdd(&W.ctr[kWsItems + cl], 1ull);
		const unsigned long long lo = atomicAdd(&W.ctr[kWsList], (unsigned long long)cnt);
		sm[35] = (u32)lo;
		sm[36] = lo + cnt <= W.list_cap ? 1u : 0u;
	}
	__syncthreads();
	const u64 it = child_begin + sm[34];
	const u32 lo = sm[35];
	const bool fits = it < W.inner.cap && sm[36];
	__syncthreads();
	if (fits) {
		const u32 k = write_child_list_block<Identity>(W, off, len, first, shift, cx, cy, cz, W.lists + lo, sm);
		if (threadIdx.x == 0) {
			W.inner.pos[it] = pack_pos(cx, cy, cz);
			W.inner.base[it] = base;
			W.inner.parent[it] = parent_slot;
			// a one-edit item holds the edit's index (written to the list by
			// this block before the barrier of the last iteration)
			W.inner.lst_off[it] = direct_edit(k) ? W.lists[lo] : lo;
			if (direct_edit(k) && cl + 2u == L)
				W.leaf_cls[it] = leaf_classes(W.edits[W.lists[lo]], cx, cy, cz);
			W.inner.lst_len[it] = k;
			if (k > W.long_threshold) {
				const unsigned long long lg = atomicAdd(&W.ctr[kWsLong + cl], 1ull);
				if (child_begin + lg < W.inner.cap)
					W.long_q[child_begin + lg] = (u32)it;
				else
					ws_error(W, kErrCapacity);
			}
		}
	} else if (threadIdx.x == 0) {
		ws_error(W, kErrCapacity);
	}
	__syncthreads();
}

// ------------------------------------------------------------------ k_expand_long
// Block per (level-l node with a long edit list, child), l <= L-3.
static __global__ void __launch_bounds__(kLongBlock) k_expand_long(DevPool P, Workspace W, u32 l) {
	apply_pass_desc(W);
	if (ws_failed(W))
		return;
	__shared__ u32 sm[40];
	const u32 L = P.cfg.L;
	const u32 cl = l + 1;
	const u64 begin = level_begin(W, L, l);
	const u64 n = W.ctr[kWsLong + l];
	const u64 child_begin = level_begin(W, L, cl);
	const u32 shift = L + 1u - cl;
	const u32 filled_c = P.cfg.filled[cl];
	for (u64 pair = blockIdx.x; pair < n * 8; pair += gridDim.x) {
		const u64 qi = begin + (pair >> 3);
		const u32 c = (u32)(pair & 7u);
		if (qi >= W.inner.cap)
			break;
		const u64 i = W.long_q[qi];
		if (i >= W.inner.cap) { // uniform over the block
			if (threadIdx.x == 0)
				ws_error(W, kErrInternal);
			break;
		}
		const u32 len = W.inner.lst_len[i], off = W.inner.lst_off[i], b = W.inner.base[i];
		const u64 pos = W.inner.pos[i];
		if (len > W.n_edits || (u64)off + len > W.list_cap) {
			if (threadIdx.x == 0)
				ws_error(W, kErrInternal);
			break;
		}
		u32 old[8];
		base_children(P, l, b, old);
		u32 cx, cy, cz;
		child_pos(pos, c, cx, cy, cz);
		u32 cb, cf;
		const u32 cnt = plan_child_block<false>(W, off, len, shift, cx, cy, cz, old[c], filled_c, &cb, &cf, sm);
		if (threadIdx.x == 0) {
			W.bchild[i * 8u + c] = old[c];
			W.cnew[i * 8u + c] = cnt ? kNull : cb;
		}
		if (cnt)
			emit_child_block<false>(W, L, cl, child_begin, (u32)(i * 8u + c), off, len, shift, cx, cy, cz, cb, cf, cnt,
			                        sm);
	}
}

// ------------------------------------------------------------------ leaf level
// New bits of the leaf at leaf coordinate (lx,ly,lz) after one edit.  A leaf
// fully covered by the edit takes the edit's value; a partially covered one
// applies the edit's 64-voxel mask (edit_leaf, NodePool.hpp:319-343).
__device__ __forceinline__ u64 apply_edit_leaf(const hd_edit_desc &e, u32 lx, u32 ly, u32 lz, u64 bits) {
	const u32 cls = classify(e, 2u, lx, ly, lz);
	if (cls == kClsNone)
		return bits;
	if (cls == kClsFull)
		return e.op == HD_OP_FILL ? ~0ull : 0ull;
	const u64 m = shape_mask(e, lx << 2, ly << 2, lz << 2);
	return e.op == HD_OP_FILL ? (bits | m) : (bits & ~m);
}

// New bits of one leaf after the edits of a list.  Inlined into the leaf
// kernels: 13 % faster than an out-of-line call.  k_leafparent_short runs 6
// blocks of 256 per SM (40 registers, the rest spilled to L1): the kernel
// waits on L2 and gains from resident warps more than it loses to the
// spills (measured on the 32768^3 batch: 3 blocks 30.1 ms, 4: 26.9, 5: 28.5,
// 6: 26.5, 7: 27.0, 8: 27.1).
__device__ __forceinline__ u64 rebuild_leaf(const Workspace &W, u32 off, u32 len, u32 lx, u32 ly, u32 lz, u64 bits) {
	for (u32 p = 0; p < len; ++p)
		bits = apply_edit_leaf(W.edits[item_list_at(W, off, len, p)], lx, ly, lz, bits);
	return bits;
}

// Result of a rebuilt leaf: unchanged / Null / filled leaf, or a dedup candidate (kNull).
__device__ __forceinline__ u32 leaf_result(const DevPool &P, u64 bits, u64 bits0, u32 old, bool *cand) {
	*cand = false;
	if (bits == bits0)
		return old;
	if (bits == 0ull)
		return kNull;
	if (bits == ~0ull)
		return P.cfg.filled[P.cfg.L - 1];
	*cand = true;
	return kNull;
}

// Read-only lookup of a leaf among the resident nodes.  No slot is pending
// while the leaves are rebuilt, so a committed entry with equal bits is the
// node; a short walk that misses leaves the leaf to the dedup launch (k_dedup).
// The walk starts at index slot s whose entry v0 the caller has loaded (the
// first slots of a node's changed leaves are loaded together).
__device__ __forceinline__ u64 leaf_slot(const DevPool &P, u64 bits) {
	return index_start(hash_leaf(bits), P.cfg.L - 1, P.index_mask);
}
__device__ __forceinline__ u32 lookup_leaf_from(const DevPool &P, u64 bits, u64 s, unsigned long long v0) {
	const u32 L = P.cfg.L, l = L - 1;
	const u32 h = hash_leaf(bits);
	const u32 bucket = P.cfg.bucket_base[l] + ((P.cfg.hasher == HD_HASHER_ZERO ? 0u : h) & ((1u << P.cfg.bucket_bits[l]) - 1u));
	const u32 bucket_shift = P.cfg.wbpp + P.cfg.pbpb;
	const u64 mask = P.index_mask;
	const unsigned long long tag = h & 0x7FFFFFFFu;
	for (u32 probe = 0; probe < 32u; ++probe, s = (s + 1) & mask) {
		const unsigned long long v = probe == 0 ? v0 : __ldg(&P.index[s]);
		if (v == kSlotEmpty)
			return kNull;
		if ((v >> 63) || ((v >> 32) & 0x7FFFFFFFull) != tag)
			continue;
		const u32 val = (u32)v;
		if ((val >> bucket_shift) != bucket)
			continue;
		const u32 *p = node_addr(P, val);
		if (p[0] == (u32)bits && p[1] == (u32)(bits >> 32))
			return val;
	}
	return kNull;
}

// Work counters of the leaf kernels, packed into two 64-bit registers per
// thread to keep the kernel within its register budget:
//   a = pairs | lookups << 24 | cache hits << 44
//   b = base-node words | old leaves << 22 | inner lookups << 43
// A thread handles at most inner.cap / (152 * 256) < 2^14 nodes, so no field
// carries into the next (pairs <= 16 per node, lookups and hits <= 8, words
// <= 9, old leaves <= 8, inner lookups <= 1).  Summed over the warp and added
// with one atomic per counter and warp; all 32 lanes call this after their
// loop.
struct LeafWork {
	u64 a = 0, b = 0;
	__device__ __forceinline__ void pairs(u32 n) { a += n; }
	__device__ __forceinline__ void lookup() { a += 1ull << 24; }
	__device__ __forceinline__ void hit() { a += 1ull << 44; }
	__device__ __forceinline__ void base_words(u32 n) { b += n; }
	__device__ __forceinline__ void old_leaf() { b += 1ull << 22; }
	__device__ __forceinline__ void inner() { b += 1ull << 43; }
};
// Read-only lookup of a changed leaf: the leaf-pattern cache first (the set's
// two slots, key and pointer side by side, in two independent 16-byte L2
// loads: one round trip; keys and pointers in separate arrays took two and
// measured 2.3 % slower), then the index; a leaf found in the index is
// entered into an empty slot of its set (key by CAS, then the pointer).
// Entries only ever name committed leaves, so a hit is exact.
__device__ __forceinline__ u32 lookup_leaf_cached(const DevPool &P, const Workspace &W, u64 bits, LeafWork &work) {
	if (!W.lc_key) {
		const u64 sl = leaf_slot(P, bits);
		return lookup_leaf_from(P, bits, sl, __ldg(&P.index[sl]));
	}
	const u32 set = hash_leaf(bits) & W.lc_mask & ~1u;
	const ulonglong2 *t = reinterpret_cast<const ulonglong2 *>(W.lc_key) + set;
	const ulonglong2 k0 = __ldcg(t), k1 = __ldcg(t + 1);
	const u32 way = k0.x == bits ? 0u : (k1.x == bits ? 1u : 2u);
	if (way < 2u) {
		const u32 v = ~(u32)(way == 0u ? k0.y : k1.y);
		if (v != kNull) {
			work.hit();
			return v;
		}
	}
	const u64 sl = leaf_slot(P, bits);
	const u32 r = lookup_leaf_from(P, bits, sl, __ldg(&P.index[sl]));
	if (r != kNull && way == 2u) {
		const u32 e = k0.x == 0ull ? 0u : (k1.x == 0ull ? 1u : 2u);
		unsigned long long *s = W.lc_key + 2u * (set + e);
		if (e < 2u && atomicCAS(s, 0ull, (unsigned long long)bits) == 0ull)
			__stcg(s + 1, (unsigned long long)(u32)~r);
	}
	return r;
}

// A level-(L-2) node whose 8 children are all known: unchanged, empty, or an
// existing node found read-only.  Returns false if it needs the dedup launch.
// The node's words (mask, then the non-null children in child order) are
// hashed and compared straight from res[], with no word array to index.
__device__ __forceinline__ bool resolve_node(const DevPool &P, u32 l, u32 base, const u32 old[8], const u32 res[8],
                                             u32 *out, LeafWork &work) {
	bool unchanged = true;
	u32 mask = 0;
#pragma unroll
	for (int c = 0; c < 8; ++c) {
		unchanged = unchanged && res[c] == old[c];
		mask |= (res[c] != kNull ? 1u : 0u) << c;
	}
	if (unchanged) {
		*out = base;
		return true;
	}
	if (!mask) {
		*out = kNull;
		return true;
	}
	Murmur mm;
	mm.add(mask);
#pragma unroll
	for (int c = 0; c < 8; ++c)
		if (res[c] != kNull)
			mm.add(res[c]);
	const u32 n = 1u + __popc(mask);
	const u32 h = mm.finish(n);
	work.inner();
	const u32 bucket = P.cfg.bucket_base[l] + ((P.cfg.hasher == HD_HASHER_ZERO ? 0u : h) & ((1u << P.cfg.bucket_bits[l]) - 1u));
	const u32 bucket_shift = P.cfg.wbpp + P.cfg.pbpb;
	const u64 imask = P.index_mask;
	const unsigned long long tag = h & 0x7FFFFFFFu;
	u64 s = index_start(h, l, imask);
	u32 r = kNull;
	for (u32 probe = 0; probe < 32u; ++probe, s = (s + 1) & imask) {
		const unsigned long long v = __ldg(&P.index[s]);
		if (v == kSlotEmpty)
			break;
		if ((v >> 63) || ((v >> 32) & 0x7FFFFFFFull) != tag)
			continue;
		const u32 val = (u32)v;
		if ((val >> bucket_shift) != bucket)
			continue;
		const u32 *p = node_addr(P, val);
		bool eq = p[0] == mask;
		u32 j = 1;
#pragma unroll
		for (int c = 0; c < 8; ++c)
			if (res[c] != kNull) {
				eq = eq && p[j] == res[c];
				++j;
			}
		if (eq) {
			r = val;
			break;
		}
	}
	*out = r;
	return r != kNull;
}

__device__ __forceinline__ void hand_to_parent(Workspace &W, u64 i, u32 r) {
	const u32 ps = W.inner.parent[i];
	if (ps == kNull)
		W.ctr[kWsRoot] = r;
	else
		W.cnew[ps] = r;
}

__device__ __forceinline__ void add_leaf_work(Workspace &W, u32 nodes, const LeafWork &w) {
	const u32 v[7] = {nodes,
	                  (u32)(w.a & 0xFFFFFFu),
	                  (u32)(w.b & 0x3FFFFFu),
	                  (u32)((w.b >> 22) & 0x1FFFFFu),
	                  (u32)((w.a >> 24) & 0xFFFFFu),
	                  (u32)(w.a >> 44),
	                  (u32)(w.b >> 43)};
#pragma unroll
	for (int k = 0; k < 7; ++k) {
		const u32 x = __reduce_add_sync(kFullMask, v[k]);
		if (lane_id() == 0 && x)
			atomicAdd(&W.ctr[kWsLeafNodes + k], (unsigned long long)x);
	}
}

// Thread per level-(L-2) node with a short edit list: computes its 8 leaves.
__device__ __forceinline__ void leafparent_short_phase(const DevPool &P, Workspace &W, u64 tbase, u64 tstride) {
	if (ws_failed(W))
		return;
	const u32 L = P.cfg.L, l = L - 2;
	u64 begin, n;
	level_range(W, L, l, begin, n);
	const u32 T = W.long_threshold;
	const u64 stride = tstride;
	u32 st_nodes = 0;
	LeafWork work;
	for (u64 w0 = tbase + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
		const u64 t = w0 + lane_id();
		const u64 i = begin + t;
		const bool valid = t < n;
		u32 len = 0, off = 0, b = kNull;
		u64 pos = 0;
		if (valid) {
			len = W.inner.lst_len[i];
			off = W.inner.lst_off[i];
			b = W.inner.base[i];
			pos = W.inner.pos[i];
		}
		const bool mine = valid && len <= T && item_list_ok(W, off, len);
		u32 old[8], res[8];
		u64 cb[8];
		u32 cand_mask = 0;
		if (mine) {
			base_children(P, l, b, old);
			st_nodes += 1;
			work.pairs(len);
			if (b != kNull && b != P.cfg.filled[l])
				work.base_words(1u + __popc(__ldg(node_addr(P, b)) & 0xFFu));
			// One edit (nearly every node): its 8 leaves classified together with
			// each axis's terms shared (classify_children, the same formulas as
			// classify per leaf), so a leaf costs a mask only when partly covered.
			const u32 e1 = len == 1u ? off : kNull; // a one-edit item holds the edit's index
			const u32 cls8 = len == 1u ? classify_children(W.edits[e1], 2u, pos_x(pos), pos_y(pos), pos_z(pos)) : 0u;
#pragma unroll 1
			for (u32 c = 0; c < 8; ++c) { // not unrolled: one copy of the leaf code keeps the i-cache warm
				u32 cx, cy, cz;
				child_pos(pos, c, cx, cy, cz);
				const u64 b0 = leaf_bits(P, old[c]);
				if (old[c] != kNull && old[c] != P.cfg.filled[L - 1])
					work.old_leaf();
				u64 bits;
				if (len == 1u) {
					const u32 cls = (cls8 >> (2u * c)) & 3u;
					const hd_edit_desc &e = W.edits[e1];
					if (cls == kClsNone)
						bits = b0;
					else if (cls == kClsFull)
						bits = e.op == HD_OP_FILL ? ~0ull : 0ull;
					else {
						const u64 m = shape_mask(e, cx << 2, cy << 2, cz << 2);
						bits = e.op == HD_OP_FILL ? (b0 | m) : (b0 & ~m);
					}
				} else {
					bits = rebuild_leaf(W, off, len, cx, cy, cz, b0);
				}
				bool cand;
				u32 r = leaf_result(P, bits, b0, old[c], &cand);
				if (cand) {
					r = lookup_leaf_cached(P, W, bits, work);
					work.lookup();
					if (r == kNull) {
						cb[c] = bits;
						cand_mask |= 1u << c;
					}
				}
				res[c] = r;
			}
		}
		// Every lane of the warp reaches both reservations below (lanes without
		// a node of their own reserve 0).
		u32 done = kNull;
		const bool resolved = mine && !cand_mask && resolve_node(P, l, b, old, res, &done, work); // no dedup round trip
		// the node's leaf candidates are contiguous, in child order
		const u64 c0 = warp_reserve(&W.ctr[kWsItems + L - 1], __popc(cand_mask));
		const u64 tq = warp_reserve(&W.ctr[kWsTodo], (mine && !resolved) ? 1u : 0u);
		if (!mine)
			continue;
		// an unresolved node's children go to its todo record: slot tq of the
		// level's own range of bchild / cnew (dense for the level-(L-2) dedup)
		const u64 ri = begin + tq;
		u64 ci = c0;
#pragma unroll 1
		for (u32 c = 0; c < 8; ++c) {
			if (!((cand_mask >> c) & 1u))
				continue;
			if (ci < W.leaf.cap) {
				W.leaf_new[ci] = cb[c];
				W.leaf.parent[ci] = (u32)(ri * 8u + c);
			} else {
				ws_error(W, kErrCapacity);
			}
			++ci;
		}
		if (resolved) {
			hand_to_parent(W, i, done);
			continue;
		}
		W.todo[tq] = (u32)i;
		W.todo_parent[tq] = W.inner.parent[i];
		uint4 *bc = reinterpret_cast<uint4 *>(W.bchild + ri * 8u);
		uint4 *cn = reinterpret_cast<uint4 *>(W.cnew + ri * 8u);
		bc[0] = make_uint4(old[0], old[1], old[2], old[3]);
		bc[1] = make_uint4(old[4], old[5], old[6], old[7]);
		cn[0] = make_uint4(res[0], res[1], res[2], res[3]);
		cn[1] = make_uint4(res[4], res[5], res[6], res[7]);
	}
	add_leaf_work(W, st_nodes, work);
}
// The same work with the deferred leaves of a warp's 32 nodes compacted onto
// all 32 lanes.  The 64-voxel mask of a partly covered leaf and its read-only
// lookup are the costly steps, and in the thread-per-node form the lanes of a
// warp reach them for different child slots, so they ran with about a third
// of the lanes active.  Here:
//   A. every lane classifies its node's 8 leaves at once (classify_children,
//      one-edit nodes) and settles the leaves the edit leaves untouched or
//      covers fully; a leaf covered partly (or fully with a resident leaf
//      under it, or any leaf of a node with several edits) is deferred;
//   B. the warp's deferred leaves (at most 256) are queued in shared memory
//      and taken 32 at a time, one per lane: rebuilt (the one edit's mask, or
//      the whole list in order), resolved (unchanged / Null / filled / found
//      by the read-only lookup), and a new leaf gets its candidate slot;
//   C. every lane takes its 8 results back and goes on as the thread-per-node
//      form does (node resolution, todo record, the candidates' parent slots).
// The per-leaf rules are the thread-per-node form's, so the results are too;
// only the order of the leaf candidates differs (a node's candidates need not
// be adjacent: each records its parent slot).
struct LeafWarpStage {
	u32 res[32 * 8];      // lane * 8 + leaf: the old child, then the leaf's result (a new leaf: its candidate slot)
	u32 old[32 * 8];      // lane * 8 + leaf: the node's old children (kept here, not in registers, across B)
	u64 pos[32];          // the lane's node
	u32 off[32], len[32], cls8[32];
	u32 cand[32];         // leaves of the lane's node that are new leaves
	unsigned char q[256]; // deferred leaves: lane << 3 | leaf
};
static constexpr int kLeafWarps = kBlock / 32;

__device__ __forceinline__ void leafparent_compact_phase(const DevPool &P, Workspace &W, u64 tbase, u64 tstride,
                                                         LeafWarpStage &S) {
	if (ws_failed(W))
		return;
	const u32 L = P.cfg.L, l = L - 2;
	u64 begin, n;
	level_range(W, L, l, begin, n);
	const u32 T = W.long_threshold;
	const u32 fl = P.cfg.filled[L - 1];
	const u64 stride = tstride;
	const u32 lane = lane_id();
	u32 st_nodes = 0;
	LeafWork work;
	for (u64 w0 = tbase + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
		const u64 t = w0 + lane;
		const u64 i = begin + t;
		const bool valid = t < n;
		u32 len = 0, off = 0, b = kNull;
		u64 pos = 0;
		if (valid) {
			len = W.inner.lst_len[i];
			off = W.inner.lst_off[i];
			b = W.inner.base[i];
			pos = W.inner.pos[i];
		}
		const bool mine = valid && len <= T && item_list_ok(W, off, len);
		u32 old[8];
		u32 defer = 0;
		// A: settle what the classification settles, defer the rest
		if (mine) {
			base_children(P, l, b, old);
			st_nodes += 1;
			work.pairs(len);
			if (b != kNull && b != P.cfg.filled[l])
				work.base_words(1u + __popc(__ldg(node_addr(P, b)) & 0xFFu));
			const u32 lc = len == 1u ? W.leaf_cls[i] : 0u; // written by the kernel that emitted the item
			const u32 cls8 = lc & 0xFFFFu;
			const bool fill = (lc >> 16) & 1u;
#pragma unroll
			for (u32 c = 0; c < 8; ++c) {
				const u32 cls = (cls8 >> (2u * c)) & 3u;
				const bool real = old[c] != kNull && old[c] != fl;
				if (real)
					work.old_leaf();
				const bool d = len != 1u || cls == kClsPartial || (cls == kClsFull && real);
				defer |= (d ? 1u : 0u) << c;
				S.res[lane * 8u + c] = (d || cls == kClsNone) ? old[c] : (fill ? fl : kNull);
			}
			S.pos[lane] = pos;
			S.off[lane] = off;
			S.len[lane] = len;
			S.cls8[lane] = cls8;
#pragma unroll
			for (u32 c = 0; c < 8; ++c)
				S.old[lane * 8u + c] = old[c];
		}
		S.cand[lane] = 0u;
		const u32 nd = __popc(defer);
		u32 incl = nd;
#pragma unroll
		for (int d = 1; d < 32; d <<= 1) {
			const u32 v = __shfl_up_sync(kFullMask, incl, d);
			if (lane >= (u32)d)
				incl += v;
		}
		const u32 total = __shfl_sync(kFullMask, incl, 31);
		u32 qpos = incl - nd;
		for (u32 m = defer; m; m &= m - 1u)
			S.q[qpos++] = (unsigned char)((lane << 3) | (u32)(__ffs(m) - 1));
		__syncwarp();
		// B: the deferred leaves, one per lane
		for (u32 j0 = 0; j0 < total; j0 += 32u) {
			const u32 j = j0 + lane;
			u32 e = 0;
			u64 nb = 0;
			bool fresh = false;
			if (j < total) {
				e = S.q[j];
				const u32 src = e >> 3, c = e & 7u;
				const u32 oldc = S.res[e], sl = S.len[src], so = S.off[src];
				u32 cx, cy, cz;
				child_pos(S.pos[src], c, cx, cy, cz);
				const u64 b0 = leaf_bits(P, oldc);
				u64 bits;
				if (sl == 1u) {
					const hd_edit_desc &ed = W.edits[so];
					if (((S.cls8[src] >> (2u * c)) & 3u) == kClsFull) {
						bits = ed.op == HD_OP_FILL ? ~0ull : 0ull;
					} else {
						const u64 m = shape_mask(ed, cx << 2, cy << 2, cz << 2);
						bits = ed.op == HD_OP_FILL ? (b0 | m) : (b0 & ~m);
					}
				} else {
					bits = rebuild_leaf(W, so, sl, cx, cy, cz, b0);
				}
				bool cand;
				u32 r = leaf_result(P, bits, b0, oldc, &cand);
				if (cand) {
					r = lookup_leaf_cached(P, W, bits, work);
					work.lookup();
					if (r == kNull) {
						fresh = true;
						nb = bits;
					}
				}
				S.res[e] = r;
			}
			// a new leaf takes its candidate slot now; its node's lane writes the parent slot
			const u64 ci = warp_reserve(&W.ctr[kWsItems + L - 1], fresh ? 1u : 0u);
			if (fresh) {
				const bool fits = ci < W.leaf.cap && ci < (u64)kNull;
				if (fits)
					W.leaf_new[ci] = nb;
				else
					ws_error(W, kErrCapacity);
				S.res[e] = fits ? (u32)ci : kNull;
				atomicOr(&S.cand[e >> 3], 1u << (e & 7u));
			}
		}
		__syncwarp();
		// C: the lane's own node
		u32 res[8];
#pragma unroll
		for (u32 c = 0; c < 8; ++c) {
			res[c] = S.res[lane * 8u + c];
			old[c] = S.old[lane * 8u + c];
		}
		const u32 cand_mask = mine ? S.cand[lane] : 0u;
		__syncwarp(); // every lane has read the stage before the next iteration rewrites it
		u32 done = kNull;
		const bool resolved = mine && !cand_mask && resolve_node(P, l, b, old, res, &done, work); // no dedup round trip
		const u64 tq = warp_reserve(&W.ctr[kWsTodo], (mine && !resolved) ? 1u : 0u);
		if (!mine)
			continue;
		const u64 ri = begin + tq;
		for (u32 m = cand_mask; m; m &= m - 1u) {
			const u32 c = (u32)(__ffs(m) - 1);
			if (res[c] != kNull)
				W.leaf.parent[res[c]] = (u32)(ri * 8u + c);
			res[c] = kNull; // written by the leaf dedup launch
		}
		if (resolved) {
			hand_to_parent(W, i, done);
			continue;
		}
		W.todo[tq] = (u32)i;
		W.todo_parent[tq] = W.inner.parent[i];
		uint4 *bc = reinterpret_cast<uint4 *>(W.bchild + ri * 8u);
		uint4 *cn = reinterpret_cast<uint4 *>(W.cnew + ri * 8u);
		bc[0] = make_uint4(old[0], old[1], old[2], old[3]);
		bc[1] = make_uint4(old[4], old[5], old[6], old[7]);
		cn[0] = make_uint4(res[0], res[1], res[2], res[3]);
		cn[1] = make_uint4(res[4], res[5], res[6], res[7]);
	}
	add_leaf_work(W, st_nodes, work);
}
static __global__ void __launch_bounds__(kBlock, 4) k_leafparent_compact(DevPool P, Workspace W) {
	__shared__ LeafWarpStage s_stage[kLeafWarps];
	apply_pass_desc(W);
	leafparent_compact_phase(P, W, (u64)blockIdx.x * blockDim.x, (u64)gridDim.x * blockDim.x,
	                         s_stage[threadIdx.x >> 5]);
}

static __global__ void __launch_bounds__(kBlock, 6) k_leafparent_short(DevPool P, Workspace W) {
	apply_pass_desc(W);
	leafparent_short_phase(P, W, (u64)blockIdx.x * blockDim.x, (u64)gridDim.x * blockDim.x);
}

// Warp per level-(L-2) node with a long edit list: lane = (leaf c = lane/4,
// quarter q = lane%4) owns voxels 16q..16q+15 of leaf c and walks the whole
// list in order.
static __global__ void __launch_bounds__(kBlock) k_leafparent_long(DevPool P, Workspace W) {
	apply_pass_desc(W);
	if (ws_failed(W))
		return;
	const u32 L = P.cfg.L, l = L - 2;
	const u64 begin = level_begin(W, L, l);
	const u64 n = W.ctr[kWsLong + l];
	const u32 lane = lane_id(), c = lane >> 2, q = lane & 3u;
	const u64 warps = (u64)gridDim.x * (blockDim.x / 32);
	u32 lw_nodes = 0;
	LeafWork work;
	for (u64 k = (u64)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; k < n; k += warps) {
		const u64 qi = begin + k;
		if (qi >= W.inner.cap)
			break;
		const u64 i = W.long_q[qi];
		if (i >= W.inner.cap) { // uniform over the warp
			if (lane == 0)
				ws_error(W, kErrInternal);
			break;
		}
		const u32 len = W.inner.lst_len[i], off = W.inner.lst_off[i], b = W.inner.base[i];
		const u64 pos = W.inner.pos[i];
		if (len > W.n_edits || (u64)off + len > W.list_cap) {
			if (lane == 0)
				ws_error(W, kErrInternal);
			break;
		}
		u32 old[8];
		base_children(P, l, b, old);
		if (lane == 0) {
			lw_nodes += 1;
			work.pairs(len);
			if (b != kNull && b != P.cfg.filled[l])
				work.base_words(1u + __popc(__ldg(node_addr(P, b)) & 0xFFu));
		}
		u32 cx, cy, cz;
		child_pos(pos, c, cx, cy, cz);
		const u64 b0 = leaf_bits(P, old[c]);
		if (q == 0 && old[c] != kNull && old[c] != P.cfg.filled[L - 1])
			work.old_leaf();
		u32 mine = (u32)(b0 >> (16u * q)) & 0xFFFFu;
		for (u32 p = 0; p < len; ++p) {
			const hd_edit_desc e = W.edits[W.lists[off + p]];
			const u32 cls = classify(e, 2u, cx, cy, cz);
			if (cls == kClsNone)
				continue;
			if (cls == kClsFull) {
				mine = e.op == HD_OP_FILL ? 0xFFFFu : 0u;
				continue;
			}
			for (u32 v = 0; v < 16; ++v) {
				const u32 iv = 16u * q + v;
				const u32 x = (cx << 2) | ((iv >> 2) & 2u) | (iv & 1u), y = (cy << 2) | ((iv >> 3) & 2u) | ((iv >> 1) & 1u),
				          z = (cz << 2) | ((iv >> 4) & 2u) | ((iv >> 2) & 1u);
				if (voxel_in(e, x, y, z))
					mine = e.op == HD_OP_FILL ? (mine | (1u << v)) : (mine & ~(1u << v));
			}
		}
		// gather the 4 quarters of each leaf
		u64 bits = 0;
#pragma unroll
		for (u32 s = 0; s < 4; ++s)
			bits |= (u64)__shfl_sync(kFullMask, mine, (lane & ~3u) | s) << (16u * s);
		const bool lead = q == 0;
		bool cand = false;
		u32 r = leaf_result(P, bits, b0, old[c], &cand);
		if (lead && cand) {
			r = lookup_leaf_cached(P, W, bits, work);
			cand = r == kNull;
			work.lookup();
		}
		cand = lead && cand;
		const u32 cmask_lanes = __ballot_sync(kFullMask, cand); // bit 4c set for candidate child c
		u32 cmask = 0;
#pragma unroll
		for (u32 k = 0; k < 8; ++k)
			cmask |= ((cmask_lanes >> (4u * k)) & 1u) << k;
		unsigned long long c0 = 0, tq = 0;
		if (lane == 0) {
			if (cmask)
				c0 = atomicAdd(&W.ctr[kWsItems + L - 1], (unsigned long long)__popc(cmask));
			tq = atomicAdd(&W.ctr[kWsTodo], 1ull);
		}
		c0 = __shfl_sync(kFullMask, c0, 0);
		tq = __shfl_sync(kFullMask, tq, 0);
		const u64 ri = begin + tq; // the node's todo record in the level's range
		if (lead) {
			if (cand) {
				const u64 ci = c0 + __popc(cmask & ((1u << c) - 1u));
				if (ci < W.leaf.cap) {
					W.leaf_new[ci] = bits;
					W.leaf.parent[ci] = (u32)(ri * 8u + c);
				} else {
					ws_error(W, kErrCapacity);
				}
			}
			W.bchild[ri * 8u + c] = old[c];
			W.cnew[ri * 8u + c] = cand ? kNull : r;
		}
		if (lane == 0) {
			W.todo[tq] = (u32)i;
			W.todo_parent[tq] = W.inner.parent[i];
		}
	}
	add_leaf_work(W, lw_nodes, work);
}

// ------------------------------------------------------------------ k_root
// NodePool.hpp:405-414 edit_switch on the root for the whole list (one block).
// With a single node level the root is a leaf and is rebuilt here directly.
__device__ __forceinline__ void root_phase(const DevPool &P, Workspace &W, u32 root_val, const u32 *root_ptr) {
	__shared__ u32 sm[40];
	const u32 L = P.cfg.L;
	const u32 root = root_ptr ? *root_ptr : root_val;
	if (threadIdx.x == 0)
		W.ctr[kWsRootIn] = root;
	// a root must be Null or point into a page that holds data
	if (root != kNull) {
		const u64 vp = root >> P.cfg.wbpp;
		const u32 phys = vp < P.total_pages ? P.page_table[vp] : kUnallocPage;
		if (phys == kUnallocPage || page_lost(P, phys)) {
			if (threadIdx.x == 0) {
				W.ctr[kWsRoot] = root;
				ws_error(W, kErrInvalidRoot);
			}
			return;
		}
	}
	if (L == 1) { // the root is a leaf: warp 0, two voxels per lane, edits in order
		if (threadIdx.x >= 32)
			return;
		const u64 b0 = leaf_bits(P, root);
		u32 v2 = (u32)(b0 >> (2u * lane_id())) & 3u;
		for (u32 p = 0; p < W.n_edits; ++p) {
			const hd_edit_desc e = W.edits[p];
#pragma unroll
			for (u32 s = 0; s < 2; ++s) {
				const u32 iv = 2u * lane_id() + s;
				const u32 x = ((iv >> 2) & 2u) | (iv & 1u), y = ((iv >> 3) & 2u) | ((iv >> 1) & 1u),
				          z = ((iv >> 4) & 2u) | ((iv >> 2) & 1u);
				if (voxel_in(e, x, y, z))
					v2 = e.op == HD_OP_FILL ? (v2 | (1u << s)) : (v2 & ~(1u << s));
			}
		}
		const u32 lo = __ballot_sync(kFullMask, v2 & 1u), hi = __ballot_sync(kFullMask, (v2 >> 1) & 1u);
		u64 bits = 0;
		for (u32 k = 0; k < 32; ++k)
			bits |= ((u64)((lo >> k) & 1u) << (2 * k)) | ((u64)((hi >> k) & 1u) << (2 * k + 1));
		if (lane_id() == 0) {
			bool cand;
			const u32 r = leaf_result(P, bits, b0, root, &cand);
			W.ctr[kWsRoot] = r;
			if (cand) { // the root leaf is the only candidate
				W.ctr[kWsItems + 0] = 1;
				W.leaf_new[0] = bits;
				W.leaf.parent[0] = kNull;
			}
		}
		return;
	}
	u32 b, f;
	const u32 cnt = plan_child_block<true>(W, 0, W.n_edits, L + 1u, 0, 0, 0, root, P.cfg.filled[0], &b, &f, sm);
	if (!cnt) {
		if (threadIdx.x == 0)
			W.ctr[kWsRoot] = b;
		return;
	}
	emit_child_block<true>(W, L, 0, 0, kNull, 0, W.n_edits, L + 1u, 0, 0, 0, b, f, cnt, sm);
}
static __global__ void __launch_bounds__(kLongBlock) k_root(DevPool P, Workspace W, u32 root_val, const u32 *root_ptr) {
	apply_pass_desc(W);
	root_phase(P, W, root_val, root_ptr);
}

// ------------------------------------------------------------------ dedup: find or insert
// One launch per level.  Every candidate is hashed, merged with the equal
// candidates of its warp, and found or inserted in the dedup index; a new node
// is written and published by the thread that claimed it, in the same launch,
// and every result goes straight into the parent's child slot.
//
// Index protocol inside a launch (later launches see only final entries and
// tombstones):
//   * a claim CAS turns an empty slot into a pending entry (bit 63, the content
//     hash tag, the claiming item);
//   * the claimer reserves its words in the bucket, writes the node, and
//     publishes the final entry with a release store -- or a tombstone when the
//     bucket is full or the heap ran out;
//   * a candidate that meets a pending entry with its tag compares its words
//     with the claiming item's words in the workspace (written by earlier
//     launches); when equal it waits for the publication and takes the pointer
//     without reading the heap;
//   * a candidate that meets a final entry with its tag has read it with an
//     acquiring CAS and compares the node through L2 (no L1 copies), so a node
//     published earlier in the same launch is seen complete.
struct NodeWords {
	u32 w[9];
	u32 n;
};

// Bounded waits: a wait that runs out records HD_ERR_TIMEOUT and fails the
// candidate instead of spinning on.
static constexpr u32 kSpinLimit = 1u << 20;

__device__ __forceinline__ unsigned long long cas_acquire(unsigned long long *p, unsigned long long cmp,
                                                          unsigned long long val) {
	unsigned long long old;
	asm volatile("atom.acquire.gpu.global.cas.b64 %0, [%1], %2, %3;" : "=l"(old) : "l"(p), "l"(cmp), "l"(val) : "memory");
	return old;
}
__device__ __forceinline__ unsigned long long load_acquire(const unsigned long long *p) {
	unsigned long long v;
	asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
	return v;
}
__device__ __forceinline__ u32 load_acquire(const u32 *p) {
	u32 v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}
__device__ __forceinline__ void store_release(unsigned long long *p, unsigned long long v) {
	asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void store_release(u32 *p, u32 v) {
	asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Physical page of virtual page vp, for a node written in this launch.  The
// thread whose reservation opened the page maps it right after its
// bucket-count CAS, so another thread that reserved words in that page in the
// same launch can find it unmapped for a moment: wait for the mapping.
__device__ __forceinline__ u32 mapped_page(const DevPool &P, u32 vp) {
	if (P.identity)
		return vp;
	u32 phys = load_acquire(P.page_table + vp);
	for (u32 spin = 0; phys == kUnallocPage; ++spin) {
		if (spin > kSpinLimit) {
			set_error(&P.counters[kCtrError], kErrTimeout);
			return kZeroPage;
		}
		__nanosleep(64);
		phys = load_acquire(P.page_table + vp);
	}
	return phys;
}

// A resident node equal to nw?  Loads through L2: the node may have been
// written earlier in this launch by another SM.
__device__ __forceinline__ bool equal_resident(const DevPool &P, u32 ptr, const NodeWords &nw) {
	const u32 *p;
	if (P.identity) {
		p = P.heap + ptr;
	} else {
		const u32 phys = __ldcg(P.page_table + (ptr >> P.cfg.wbpp));
		p = P.heap + ((u64)phys << P.cfg.wbpp) + (ptr & (wpp(P.cfg) - 1u));
	}
	for (u32 k = 0; k < nw.n; ++k)
		if (__ldcg(p + k) != nw.w[k])
			return false;
	return true;
}

// Reserve space for a node of w words in bucket b (NodePool.hpp:134-157 on an
// atomic word count).  Returns false when the bucket is full.  *pad_out is the
// old word count when the node skips the rest of a page (that tail must be
// zeroed), else kNull.
__device__ __forceinline__ bool reserve(const DevPool &P, u32 b, u32 w, u32 *ptr_out, u32 *pad_out, u32 *retries) {
	const u32 wp = wpp(P.cfg), wpb = 1u << (P.cfg.wbpp + P.cfg.pbpb);
	u32 old = *(volatile u32 *)&P.bucket_words[b];
	u32 off, nw;
	for (u32 tries = 0;; ++tries) { // lock-free: a failed CAS means another thread advanced the count
		if (tries > (1u << 22)) {  // cannot happen with fewer than 2^22 contenders; report, do not spin
			set_error(&P.counters[kCtrError], kErrTimeout);
			return false;
		}
		off = old;
		if ((off & (wp - 1u)) + w > wp)
			off = (off | (wp - 1u)) + 1u;
		nw = off + w;
		if (nw > wpb)
			return false;
		const u32 prev = atomicCAS(&P.bucket_words[b], old, nw);
		if (prev == old)
			break;
		++*retries;
		old = prev;
	}
	*pad_out = off != old ? old : kNull;
	const u32 vpage = (b << P.cfg.pbpb) | (off >> P.cfg.wbpp);
	if ((off & (wp - 1u)) == 0u) { // this node opens the page
		u32 phys = atomicAdd(&P.counters[kCtrHeapNext], 1u);
		if (P.identity)
			phys = vpage;
		else if (phys >= P.heap_pages) {
			phys = kZeroPage;
			set_error(&P.counters[kCtrError], kErrOom);
		}
		if (!P.identity)
			store_release(P.page_table + vpage, phys);
		else
			P.page_table[vpage] = phys;
	}
	*ptr_out = (b << (P.cfg.wbpp + P.cfg.pbpb)) | off;
	return true;
}

// Writes a reserved node, and zeroes the page tail its reservation skipped
// (NodePool.hpp:145-150).  False if its page could not be allocated.
__device__ __forceinline__ bool write_node(const DevPool &P, u32 ptr, u32 pad, const NodeWords &nw) {
	const u32 wp = wpp(P.cfg);
	const u32 phys = mapped_page(P, ptr >> P.cfg.wbpp);
	if (page_lost(P, phys))
		return false;
	u32 *dst = P.heap + ((u64)phys << P.cfg.wbpp) + (ptr & (wp - 1u));
	for (u32 k = 0; k < nw.n; ++k)
		dst[k] = nw.w[k];
	if (pad != kNull) {
		const u32 vp = ((ptr >> (P.cfg.wbpp + P.cfg.pbpb)) << P.cfg.pbpb) | (pad >> P.cfg.wbpp);
		const u32 zp = mapped_page(P, vp);
		if (!page_lost(P, zp)) {
			u32 *z = P.heap + ((u64)zp << P.cfg.wbpp);
			for (u32 q = pad & (wp - 1u); q < wp; ++q)
				z[q] = 0u;
		}
	}
	return true;
}

// Pointer published in slot s by the thread that claimed it in this launch,
// or kNull when that insertion failed (its error is already recorded).
__device__ __forceinline__ u32 await_publication(const DevPool &P, u64 s) {
	for (u32 spin = 0;; ++spin) {
		const unsigned long long v = load_acquire(&P.index[s]);
		if (v == kSlotTomb)
			return kNull;
		if (!(v >> 63))
			return (u32)v;
		if (spin > kSpinLimit) {
			set_error(&P.counters[kCtrError], kErrTimeout);
			return kNull;
		}
		__nanosleep(32);
	}
}

// Find-or-insert of one candidate (NodePool.hpp:159-212 upsert_node with the
// linear bucket scan replaced by the index).  cmp_pending(j) tests equality
// with the words of item j of this level.  The probe walks at most kMaxProbe
// slots (a table at its load limit needs a few dozen); a longer walk is
// reported as a full index instead of scanned.  Returns the node's pointer, or
// kNull when the insertion failed (error recorded).
static constexpr u64 kMaxProbe = 1u << 16;
template <typename CmpPending>
__device__ __forceinline__ u32 find_or_insert(const DevPool &P, u64 i, u32 level, u32 h, u32 bucket,
                                              const NodeWords &nw, u32 *probes, u32 *retries, bool *inserted,
                                              CmpPending &&cmp_pending) {
	const u64 mask = P.index_mask;
	const unsigned long long tag = (unsigned long long)(h & 0x7FFFFFFFu) << 32;
	const u32 bucket_shift = P.cfg.wbpp + P.cfg.pbpb;
	const u64 limit = mask < kMaxProbe ? mask + 1 : kMaxProbe;
	u64 s = index_start(h, level, mask);
	const unsigned long long claim = (1ull << 63) | tag | (unsigned long long)i;
	u32 r = kNull;
	*inserted = false;
	u64 probe = 0;
	for (; probe < limit; ++probe, s = (s + 1) & mask) {
		// claim-or-read in one atomic: an empty slot is claimed at once, an
		// occupied one returns its entry
		const unsigned long long v = cas_acquire(&P.index[s], kSlotEmpty, claim);
		if (v == kSlotEmpty) {
			u32 ptr, pad;
			if (!reserve(P, bucket, nw.n, &ptr, &pad, retries)) {
				set_error(&P.counters[kCtrError], kErrBucketFull);
				store_release(&P.index[s], kSlotTomb);
			} else if (!write_node(P, ptr, pad, nw)) {
				set_error(&P.counters[kCtrError], kErrOom);
				store_release(&P.index[s], kSlotTomb);
			} else {
				store_release(&P.index[s], tag | ptr);
				r = ptr;
				*inserted = true;
			}
			break;
		}
		if (v == kSlotTomb || (v & (0x7FFFFFFFull << 32)) != tag)
			continue;
		if (v >> 63) { // claimed in this launch by item (u32)v
			if (!cmp_pending((u32)v))
				continue;
			r = await_publication(P, s);
			break;
		}
		const u32 val = (u32)v;
		if ((val >> bucket_shift) == bucket && equal_resident(P, val, nw)) {
			r = val;
			break;
		}
	}
	if (probe == limit)
		set_error(&P.counters[kCtrError], kErrIndexFull);
	*probes = (u32)probe + 1u;
	return r;
}

// Per-thread statistics summed (or maxed) over the warp and added to the
// block's shared accumulators; the block's last warp to get here adds them to
// the global counters (one global atomic per counter and block instead of one
// per warp and iteration).  No block barrier: warps that finish early leave at
// once instead of waiting for the block's slowest warp.  s_acc (N slots) and
// *s_done are zeroed before the block's first __syncthreads; every warp of the
// block calls this once, with all its lanes, after its loop.
template <int N>
__device__ __forceinline__ void flush_block_stats(const unsigned long long (&v)[N], unsigned long long *const (&dst)[N],
                                                  const bool (&is_max)[N], unsigned long long *s_acc, u32 *s_done) {
#pragma unroll
	for (int k = 0; k < N; ++k) {
		unsigned long long x = v[k];
#pragma unroll
		for (int d = 16; d > 0; d >>= 1) {
			const unsigned long long y = __shfl_down_sync(kFullMask, x, d);
			x = is_max[k] ? (x > y ? x : y) : x + y;
		}
		if (lane_id() == 0 && x) {
			if (is_max[k])
				atomicMax(&s_acc[k], x);
			else
				atomicAdd(&s_acc[k], x);
		}
	}
	u32 last = 0;
	if (lane_id() == 0) {
		__threadfence_block();
		last = atomicAdd(s_done, 1u) == (blockDim.x >> 5) - 1u ? 1u : 0u;
	}
	if (!__shfl_sync(kFullMask, last, 0))
		return;
	__threadfence_block();
	if (lane_id() < (u32)N) {
		const u32 k = lane_id();
		const unsigned long long x = atomicAdd(&s_acc[k], 0ull); // read after every warp's update
		if (x) {
			if (is_max[k])
				atomicMax(dst[k], x);
			else
				atomicAdd(dst[k], x);
		}
	}
}

// ------------------------------------------------------------------ k_dedup
// Leaf: the leaf candidates.  Inner: the level-l items, rebuilt from cnew.
// Leaves repeat a few patterns many times: each block keeps a direct-mapped
// shared-memory cache of leaf bits -> pointer for leaves found resident, so
// repeated patterns are answered without touching the index.
static constexpr u32 kLeafCache = 2048;
// Item t of a level: position t of the level range, or for level L-2 the
// t-th todo record (slot t of the level's range of bchild / cnew, written by
// the leaf kernel; the node itself is W.todo[t]).
__device__ __forceinline__ u64 item_at(const Workspace &W, u32 use_todo, u64 begin, u64 t) {
	return begin + t;
}
__device__ __forceinline__ void dedup_range(const Workspace &W, u32 L, u32 l, u32 use_todo, u64 &begin, u64 &n) {
	level_range(W, L, l, begin, n);
	if (use_todo) {
		const u64 nt = W.ctr[kWsTodo];
		n = nt < n ? nt : n;
	}
}
__device__ __forceinline__ u32 sat_add(u32 a, u32 b) { return a + b < a ? 0xFFFFFFFFu : a + b; }

template <bool Leaf>
__device__ __forceinline__ void dedup_phase(const DevPool &P, Workspace &W, u32 l, u32 use_todo, u64 tbase,
                                            u64 tstride) {
	if (ws_failed(W))
		return;
	__shared__ int s_skip;
	__shared__ unsigned long long s_key[Leaf ? kLeafCache : 1];
	__shared__ u32 s_val[Leaf ? kLeafCache : 1];
	if (Leaf)
		for (u32 e = threadIdx.x; e < kLeafCache; e += blockDim.x) {
			s_key[e] = 0ull; // empty slot (all-zero leaves are never cached)
			s_val[e] = kNull;
		}
	__shared__ unsigned long long s_acc[7];
	__shared__ u32 s_done;
	if (threadIdx.x < 7)
		s_acc[threadIdx.x] = 0ull;
	if (threadIdx.x == 0) {
		s_skip = pool_failed(P) ? 1 : 0;
		s_done = 0u;
	}
	__syncthreads();
	const bool skip = s_skip != 0; // an earlier level failed: insert nothing more, hand Null up
	// per-thread sums (saturating)
	u32 a_cand = 0, a_words = 0, a_steps = 0, a_retry = 0, a_max = 0, a_ins = 0, a_insw = 0;
	const u32 L = P.cfg.L;
	u64 begin, n;
	dedup_range(W, L, l, use_todo, begin, n);
	Items &it = Leaf ? W.leaf : W.inner;
	const u32 nb_mask = (1u << P.cfg.bucket_bits[l]) - 1u;
	const u32 bbase = P.cfg.bucket_base[l];
	const bool zero_hash = P.cfg.hasher == HD_HASHER_ZERO;
	const u32 lane = lane_id();
	const u64 stride = tstride;
	for (u64 w0 = tbase + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
		const u64 t = w0 + lane;
		const bool valid = t < n;
		const u64 i = valid ? item_at(W, use_todo, begin, t) : 0;
		bool cand = false;
		u32 r = kNull;
		NodeWords nw;
		nw.n = 0;
#pragma unroll
		for (int k = 0; k < 9; ++k)
			nw.w[k] = 0;
		u32 h = 0;
		if (valid && !skip) {
			if (Leaf) {
				const u64 bits = W.leaf_new[i];
				nw.w[0] = (u32)bits;
				nw.w[1] = (u32)(bits >> 32);
				nw.n = 2;
				h = hash_leaf(bits);
				cand = true;
			} else {
				const uint4 *cn4 = reinterpret_cast<const uint4 *>(W.cnew + i * 8u);
				const uint4 *bc4 = reinterpret_cast<const uint4 *>(W.bchild + i * 8u);
				const uint4 a0 = cn4[0], a1 = cn4[1];
				const uint4 b0 = bc4[0], b1 = bc4[1];
				const u32 c[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
				if (a0.x == b0.x && a0.y == b0.y && a0.z == b0.z && a0.w == b0.w && a1.x == b1.x && a1.y == b1.y &&
				    a1.z == b1.z && a1.w == b1.w) {
					r = it.base[use_todo ? (u64)W.todo[t] : i]; // no child changed
				} else {
					u32 mask = 0, k = 1;
#pragma unroll
					for (int q = 0; q < 8; ++q)
						if (c[q] != kNull) {
							mask |= 1u << q;
							nw.w[k++] = c[q];
						}
					if (mask) { // else every child is gone: Null
						nw.w[0] = mask;
						nw.n = k;
						Murmur mm;
						for (u32 q = 0; q < k; ++q)
							mm.add(nw.w[q]);
						h = mm.finish(k);
						cand = true;
					}
				}
			}
		}
		// cached leaf: found without a probe
		bool hit = false;
		u32 slot_e = 0;
		// key 0 marks an empty cache slot, so an all-zero leaf (possible only
		// through the upsert calls) is never cached and always probes
		const bool cacheable = Leaf && cand && (nw.w[0] | nw.w[1]) != 0u;
		if (cacheable) {
			const u64 bits = (u64)nw.w[0] | ((u64)nw.w[1] << 32);
			slot_e = (h ^ (h >> 13)) & (kLeafCache - 1u);
			if (s_key[slot_e] == bits) {
				const u32 hp = *(volatile u32 *)&s_val[slot_e];
				if (hp != kNull) {
					hit = true;
					r = hp;
				}
			}
		}
		const bool probe_me = cand && !hit;
		// merge equal candidates of the warp: one leader probes, the others follow
		const unsigned long long key = probe_me ? (unsigned long long)h : (0x100000000ull | lane);
		const u32 same = __match_any_sync(kFullMask, key);
		const u32 leader = __ffs(same) - 1u;
		// every lane executes every shuffle (no short-circuit around a full-mask shuffle)
		const u32 leader_n = __shfl_sync(kFullMask, nw.n, leader);
		bool eq = probe_me && leader != lane && leader_n == nw.n;
#pragma unroll
		for (int k = 0; k < 9; ++k) {
			const u32 lw = __shfl_sync(kFullMask, nw.w[k], leader);
			eq = eq && lw == nw.w[k];
		}
		const bool follower = eq;
		u32 probes = 0, retries = 0, mine = kNull;
		bool ins = false;
		if (probe_me && !follower) {
			const u32 bucket = bbase + ((zero_hash ? 0u : h) & nb_mask);
			if (Leaf) {
				const u64 bits = (u64)nw.w[0] | ((u64)nw.w[1] << 32);
				mine = find_or_insert(P, i, l, h, bucket, nw, &probes, &retries, &ins,
				                      [&](u32 j) { return W.leaf_new[j] == bits; });
			} else {
				mine = find_or_insert(P, i, l, h, bucket, nw, &probes, &retries, &ins, [&](u32 j) {
					const uint4 *o4 = reinterpret_cast<const uint4 *>(W.cnew + (u64)j * 8u);
					const uint4 c0 = o4[0], c1 = o4[1];
					u32 m = 0, k = 1;
					const u32 c[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
					bool same_words = true;
#pragma unroll
					for (int q = 0; q < 8; ++q)
						if (c[q] != kNull) {
							m |= 1u << q;
							same_words = same_words && k < nw.n && c[q] == nw.w[k];
							++k;
						}
					return same_words && m == nw.w[0] && k == nw.n;
				});
			}
		}
		const u32 lres = __shfl_sync(kFullMask, mine, leader);
		if (probe_me)
			r = follower ? lres : mine;
		if (cacheable && probe_me && !follower && !ins && r != kNull) { // found resident: remember it in the block
			const u64 bits = (u64)nw.w[0] | ((u64)nw.w[1] << 32);
			if (s_key[slot_e] == 0ull && atomicCAS(&s_key[slot_e], 0ull, (unsigned long long)bits) == 0ull)
				*(volatile u32 *)&s_val[slot_e] = r;
		}
		if (valid) {
			const u32 ps = use_todo ? W.todo_parent[t] : it.parent[i];
			if (ps == kNull) { // the pass's root item, or a node of an upsert call
				W.ctr[kWsRoot] = r;
				it.res[i] = r;
			} else {
				W.cnew[ps] = r;
			}
		}
		a_cand += cand ? 1u : 0u;
		a_words += cand ? nw.n : 0u;
		a_ins += ins ? 1u : 0u;
		a_insw += ins ? nw.n : 0u;
		a_steps = sat_add(a_steps, probes);
		a_retry = sat_add(a_retry, retries);
		a_max = a_max > probes ? a_max : probes;
	}
	const unsigned long long v[7] = {a_cand, a_words, a_steps, a_retry, a_max, a_ins, a_insw};
	unsigned long long *const dst[7] = {&W.ctr[kWsCand + l], &W.ctr[kWsCandWords + l], &W.ctr[kWsProbeSteps],
	                                    &W.ctr[kWsCasRetry],  &W.ctr[kWsMaxProbe],     &W.ctr[kWsIns + l],
	                                    &W.ctr[kWsInsWords + l]};
	const bool is_max[7] = {false, false, false, false, true, false, false};
	flush_block_stats(v, dst, is_max, s_acc, &s_done);
}
template <bool Leaf>
static __global__ void __launch_bounds__(kBlock) k_dedup(DevPool P, Workspace W, u32 l, u32 use_todo) {
	apply_pass_desc(W);
	dedup_phase<Leaf>(P, W, l, use_todo, (u64)blockIdx.x * blockDim.x, (u64)gridDim.x * blockDim.x);
}

// ------------------------------------------------------------------ k_finish
__device__ __forceinline__ void finish_phase(const DevPool &P, Workspace &W, u32 *out_root) {
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
static __global__ void k_finish(DevPool P, Workspace W, u32 *out_root) { finish_phase(P, W, out_root); }

// ------------------------------------------------------------------ one-CTA pass
// A whole pass in one block, the phases separated by block barriers instead of
// kernel boundaries: the plain one-edit form (and other small passes) costs one
// launch.  Only for passes without long edit lists (n_edits <= long_threshold),
// whose every list is handled by the short phases.  Between phases a thread
// reads what other threads of the block wrote before the barrier; the
// read-only loads (index lookups in the leaf phase, page-table reads) never
// touch words written earlier in the same pass.
static __global__ void __launch_bounds__(kBlock) k_small_pass(DevPool P, Workspace W, u32 root_val, const u32 *root_ptr,
                                                              u32 *out_root) {
	const u32 L = P.cfg.L;
	const u64 tb = 0, ts = blockDim.x;
	root_phase(P, W, root_val, root_ptr);
	__syncthreads();
	for (u32 l = 0; l + 2 < L; ++l) {
		expand_short_phase<false>(P, W, l, tb, ts);
		__syncthreads();
	}
	if (L >= 2) {
		leafparent_short_phase(P, W, tb, ts);
		__syncthreads();
	}
	dedup_phase<true>(P, W, L - 1, 0u, tb, ts);
	__syncthreads();
	for (u32 l = L - 1; l-- > 0;) {
		const u32 todo = l + 2 == L ? 1u : 0u; // level L-2 runs over the unresolved nodes only
		dedup_phase<false>(P, W, l, todo, tb, ts);
		__syncthreads();
	}
	finish_phase(P, W, out_root);
}

} // namespace hd
