// hd_color.cu -- colour (VBR) editing and colour lookup on the device.
//
// Replaces the application's colour octree DAGColorPool
// (src/DAGColorPool.hpp:20-218) and colour editing through
// hashdag::VBREditorWrapper (include/hashdag/VBREditor.hpp:26-107) with the
// VBR chunk writer of include/hashdag/VBRColor.hpp:367-488, plus the colour
// fetch of trace.frag:272-356.  The pool words (octree nodes, leaf blocks)
// are the ones the reference's single-threaded NodePoolBase::Edit writes.
//
// Layout (the application's, src/DAGColorPool.hpp:22-60): a pointer is a
// 2-bit tag (0 node, 1 colour, 2 leaf, 3 null) over 30 bits of data (node
// index, RGB8 colour, leaf word index).  Nodes are 8 pointers.  A leaf block is
// [block size][macro count M][block count B][weight word count W]
// [M macro blocks: first block, weight start][B block headers: colours,
// voxel offset:14 | bits per weight:2 | weight offset:16][W weight words].
// A colour leaf covers the 8^(voxel_level - leaf_level) voxels under an octree
// node at leaf_level in Morton order (NodeCoord.hpp:18-43 child and leaf
// voxel order); a macro block spans 2^14 of them.
//
// One colour edit (the colour part of a VBR fill or paint):
//   k_color_walk   one CTA walks the octree from the root down to leaf_level
//                  against the OLD DAG (the wrapper's EditNode colour rules):
//                  a node the edit covers, whose DAG node is empty or whose
//                  fill colour is the edit's becomes the edit's colour; an
//                  untouched node stays; a partly covered leaf-level node
//                  becomes a region whose chunk is rewritten
//   k_color_count  CTA per region: per DAG-leaf unit (64 voxels) of the
//                  region its new colours (the first DAG node on the way down
//                  that the edit covers or that is empty gives the edit's
//                  colour, the first one it does not touch keeps the old
//                  colours, else per voxel: the edit's colour if the voxel is
//                  in the shape or was empty); block and weight-bit counts
//   k_color_place  one CTA: chunk sizes -> scratch offsets, in-place rewrite
//                  or append (SetLeaf, src/DAGColorPool.hpp:176-207) in
//                  region (= JoinNode) order
//   k_color_emit   CTA per region: the chunk into scratch (the old chunk may
//                  be the destination of an in-place rewrite)
//   k_color_copy   CTA per region: scratch -> leaf blocks
//   k_color_up     one CTA: SetNode bottom-up (src/DAGColorPool.hpp:150-165);
//                  appended nodes numbered in JoinNode (post) order
// The geometry of a fill then goes through hd_edit (paint keeps it).
#include "hd_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#define HD_TRY(x)                                                                                                     \
	do {                                                                                                              \
		cudaError_t e_ = (x);                                                                                         \
		if (e_ != cudaSuccess) {                                                                                      \
			fprintf(stderr, "hashdag_gb300: %s failed: %s\n", #x, cudaGetErrorString(e_));                           \
			return HD_ERR_CUDA;                                                                                       \
		}                                                                                                             \
	} while (0)

using namespace hd;

namespace {

constexpr u32 kTagNode = 0, kTagColor = 1, kTagLeaf = 2, kTagNull = 3;
constexpr u32 kCNull = kTagNull << 30;
constexpr u32 kMacroBits = 14; // VBRInfo::kVoxelBitsPerMacroBlock
constexpr u32 kMacroVoxels = 1u << kMacroBits;
constexpr u32 kUnitsPerMacro = kMacroVoxels / 64u;
constexpr int kWalkBlock = 1024;
constexpr int kRegionBlock = 256; // one macro block of DAG-leaf units per iteration
static_assert(kRegionBlock == (int)kUnitsPerMacro, "region kernels process one macro block per iteration");

// walk decisions
enum : u32 { kDecKeep = 0, kDecFill = 1, kDecProceed = 2, kDecRegion = 3 };
// device error codes of a colour edit
enum : u32 { kCErrNone = 0, kCErrItems = 1, kCErrNodes = 2, kCErrLeaves = 3, kCErrScratch = 4 };

__host__ __device__ __forceinline__ u32 ctag(u32 p) { return p >> 30; }
__host__ __device__ __forceinline__ u32 cdata(u32 p) { return p & 0x3FFFFFFFu; }
__host__ __device__ __forceinline__ u32 cptr(u32 tag, u32 data) { return (tag << 30) | data; }

struct VCol { // VBRColor (VBRColor.hpp:18-43)
	u32 colors, weight, bpw, has;
};

// VBRColor::Get (VBRColor.hpp:31-36): RGB8Color / R5G6B5Color::Get
// (Color.hpp:24,42-45) and mix = x * (1 - a) + y * a, every step rounded
// separately (no contraction) as the reference computes it.
__host__ __device__ __forceinline__ float fdiv(float a, float b) {
#ifdef __CUDA_ARCH__
	return __fdiv_rn(a, b);
#else
	return a / b;
#endif
}
__host__ __device__ __forceinline__ float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
	return __fmul_rn(a, b);
#else
	return a * b;
#endif
}
__host__ __device__ __forceinline__ float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
	return __fadd_rn(a, b);
#else
	return a + b;
#endif
}
__host__ __device__ __forceinline__ float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
	return __fsub_rn(a, b);
#else
	return a - b;
#endif
}
__host__ __device__ __forceinline__ void vcol_rgb(const VCol &c, float rgb[3]) {
	if (c.bpw == 0) {
		for (int k = 0; k < 3; ++k)
			rgb[k] = fdiv((float)((c.colors >> (8 * k)) & 0xFFu), 255.0f);
		return;
	}
	const u32 lo = c.colors & 0xFFFFu, hi = c.colors >> 16;
	const float x[3] = {fdiv((float)(lo & 0x1Fu), 31.0f), fdiv((float)((lo >> 5) & 0x3Fu), 63.0f),
	                    fdiv((float)((lo >> 11) & 0x1Fu), 31.0f)};
	const float y[3] = {fdiv((float)(hi & 0x1Fu), 31.0f), fdiv((float)((hi >> 5) & 0x3Fu), 63.0f),
	                    fdiv((float)((hi >> 11) & 0x1Fu), 31.0f)};
	const float a = fdiv((float)c.weight, (float)((1u << c.bpw) - 1u));
	const float one_minus = fsub(1.0f, a);
	for (int k = 0; k < 3; ++k)
		rgb[k] = fadd(fmul(x[k], one_minus), fmul(y[k], a));
}
// DAGColorPool::FillNode (src/DAGColorPool.hpp:167-169): RGB8Color{color.Get()}
__host__ __device__ __forceinline__ u32 vcol_rgb8(const VCol &c) {
	float rgb[3];
	vcol_rgb(c, rgb);
	u32 out = 0;
	for (int k = 0; k < 3; ++k)
		out |= ((u32)(unsigned char)(fmul(rgb[k], 255.0f))) << (8 * k);
	return out;
}

struct ColorDev {
	u32 *nodes;                // [max_nodes * 8]
	u32 *leaves;               // [max_leaf_words]
	unsigned long long *ctr;   // [0] nodes, [1] leaf words
	unsigned long long max_nodes, max_leaf_words;
	u32 leaf_level, keep_history;
};

// per-edit workspace (device)
struct ColorWs {
	// walk items of levels 0..leaf_level, level by level; lvl[l] = first item of level l, lvl[LL+1] = total
	u64 *pos;  // packed coordinate at the item's level
	u32 *optr; // old octree pointer
	u32 *dptr; // old DAG node
	u32 *res;  // new octree pointer
	u32 *dec;  // walk decision
	u32 *child; // first child item (kDecProceed) / region index (kDecRegion)
	u32 *app;  // 1: the node is appended (k_color_up)
	u32 *nidx; // appended node index
	u64 item_cap;
	u32 *lvl;      // [HD_MAX_LEVELS + 2]
	u32 *regions;  // region -> item
	u32 *r_words;  // chunk words (without the block size word)
	u64 *r_blocks; // block headers of the chunk
	u64 *r_scratch; // scratch offset
	u64 *r_dest;   // leaf word index of the block
	u64 *r_append; // appended words (0: rewritten in place)
	u64 region_cap;
	// per (region, macro block) q = region * macros + macro: block headers and
	// weight bits of the macro block, then their offsets inside the chunk
	u64 *m_blocks, *m_bits, *m_hoff, *m_boff;
	u32 macros; // macro blocks per colour leaf
	u32 *scratch;
	u64 scratch_cap;
	u32 *app_list; // appended items, level by level in Morton order
	u32 *app_lvl;  // [HD_MAX_LEVELS + 2]
	u64 *app_end;  // end position of each listed item (leaf-level Morton units)
	// [0] regions, [1] scratch words needed, [2] leaf words appended, [3] error,
	// [4] new colour root, [5] nodes appended
	unsigned long long *c;
};

struct EditArgs {
	hd_edit_desc e; // op FILL geometry
	VCol C;
	u32 rgb8;       // FillNode colour of C
	u32 root, color_root;
};

__device__ __forceinline__ u64 pk(u32 x, u32 y, u32 z) { return (u64)x | ((u64)y << 21) | ((u64)z << 42); }
__device__ __forceinline__ void upk(u64 p, u32 &x, u32 &y, u32 &z) {
	x = (u32)(p & 0x1FFFFFu);
	y = (u32)((p >> 21) & 0x1FFFFFu);
	z = (u32)((p >> 42) & 0x1FFFFFu);
}

// child c of an inner DAG node (NodePool.hpp:278-309)
__device__ __forceinline__ u32 dag_child(const DevPool &P, u32 node, u32 c) {
	if (node == kNull)
		return kNull;
	const u32 *p = node_addr(P, node);
	const u32 m = p[0] & 0xFFu;
	return ((m >> c) & 1u) ? p[1 + __popc(m & ((1u << c) - 1u))] : kNull;
}

__device__ __forceinline__ VCol fill_of(u32 p) { return ctag(p) == kTagColor ? VCol{cdata(p), 0, 0, 1} : VCol{0, 0, 0, 0}; }
__device__ __forceinline__ bool vcol_eq(const VCol &a, const VCol &b) {
	return a.colors == b.colors && a.weight == b.weight && a.bpw == b.bpw && a.has == b.has;
}
// DAGColorPool::GetChild (src/DAGColorPool.hpp:142-146)
__device__ __forceinline__ u32 octree_child(const ColorDev &C, u32 p, u32 c) {
	return ctag(p) == kTagNode ? C.nodes[(u64)cdata(p) * 8u + c] : (ctag(p) == kTagColor ? p : kCNull);
}

// Exclusive scan over the block (blockDim.x a multiple of 32, <= 1024); *total = sum.
__device__ __forceinline__ u64 block_scan(u64 v, u64 *s_warp, u64 *total) {
	const u32 lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	u64 incl = v;
	for (int d = 1; d < 32; d <<= 1) {
		const u64 t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
		if (lane >= (u32)d)
			incl += t;
	}
	if (lane == 31)
		s_warp[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		u64 w = lane < nw ? s_warp[lane] : 0ull, wi = w;
		for (int d = 1; d < 32; d <<= 1) {
			const u64 t = __shfl_up_sync(0xFFFFFFFFu, wi, d);
			if (lane >= (u32)d)
				wi += t;
		}
		if (lane < nw)
			s_warp[lane] = wi - w;
		if (lane == 31)
			s_warp[32] = wi;
	}
	__syncthreads();
	const u64 r = s_warp[warp] + incl - v;
	*total = s_warp[32];
	__syncthreads();
	return r;
}

// ------------------------------------------------------------------ walk
// VBREditorWrapper::EditNode at and above leaf_level (VBREditor.hpp:40-80)
// with the editors' colour rules (src/main.cpp:48-58,107-127).
__global__ void __launch_bounds__(kWalkBlock) k_color_walk(DevPool P, ColorDev C, ColorWs W, EditArgs a) {
	__shared__ u64 s_warp[33];
	const u32 LL = C.leaf_level, V = P.cfg.L + 1u;
	if (threadIdx.x == 0) {
		W.lvl[0] = 0;
		W.lvl[1] = 1;
		W.pos[0] = 0;
		W.optr[0] = a.color_root;
		W.dptr[0] = a.root;
		W.c[0] = 0;
	}
	__syncthreads();
	u64 n_regions = 0;
	for (u32 l = 0; l <= LL; ++l) {
		const u32 b = W.lvl[l], e = W.lvl[l + 1];
		u64 next = e; // first item of level l+1
		for (u32 i0 = b; i0 < e; i0 += blockDim.x) {
			const u32 i = i0 + threadIdx.x;
			u32 dec = kDecKeep;
			if (i < e) {
				u32 x, y, z;
				upk(W.pos[i], x, y, z);
				const u32 cls = classify(a.e, V - l, x, y, z);
				const u32 o = W.optr[i];
				if (cls == kClsFull || W.dptr[i] == kNull || vcol_eq(fill_of(o), a.C)) {
					dec = kDecFill;
					W.res[i] = cptr(kTagColor, a.rgb8);
				} else if (cls == kClsNone) {
					W.res[i] = o;
				} else {
					dec = l == LL ? kDecRegion : kDecProceed;
				}
				W.dec[i] = dec;
				W.app[i] = 0;
			}
			u64 tot;
			const u64 rank = block_scan(dec == kDecProceed ? 1u : 0u, s_warp, &tot);
			u64 rtot;
			const u64 rrank = block_scan(dec == kDecRegion ? 1u : 0u, s_warp, &rtot);
			if (dec == kDecProceed) {
				const u64 c0 = next + 8ull * rank;
				if (c0 + 8 <= W.item_cap) {
					W.child[i] = (u32)c0;
					u32 x, y, z;
					upk(W.pos[i], x, y, z);
					const u32 o = W.optr[i], d = W.dptr[i];
					for (u32 c = 0; c < 8; ++c) {
						W.pos[c0 + c] = pk((x << 1) | (c & 1u), (y << 1) | ((c >> 1) & 1u), (z << 1) | ((c >> 2) & 1u));
						W.optr[c0 + c] = octree_child(C, o, c);
						W.dptr[c0 + c] = dag_child(P, d, c);
					}
				} else {
					atomicCAS(&W.c[3], 0ull, (unsigned long long)kCErrItems);
				}
			}
			if (dec == kDecRegion) {
				const u64 r = n_regions + rrank;
				if (r < W.region_cap) {
					W.regions[r] = i;
					W.child[i] = (u32)r;
				} else {
					atomicCAS(&W.c[3], 0ull, (unsigned long long)kCErrItems);
				}
			}
			next += 8ull * tot;
			n_regions += rtot;
		}
		if (threadIdx.x == 0)
			W.lvl[l + 2] = (u32)(next < W.item_cap ? next : W.item_cap);
		__syncthreads();
		if (*(volatile unsigned long long *)&W.c[3]) // out of room: the next level's items were not all written
			break;
	}
	if (threadIdx.x == 0)
		W.c[0] = n_regions < W.region_cap ? n_regions : W.region_cap;
}

// ------------------------------------------------------------------ regions
struct Region {
	u32 dptr, optr;
	u32 x, y, z;     // region coordinate at leaf_level
	u32 units;       // DAG-leaf units (64 voxels each)
	u32 unit_levels; // levels from leaf_level down to the DAG leaf level
	// old chunk (has_src) or the fill colour
	bool has_src;
	const u32 *macro, *hdr, *bits;
	u32 M, B, W;
	VCol fill;
};

__device__ __forceinline__ Region region_of(const DevPool &P, const ColorDev &C, const ColorWs &W, u32 r) {
	Region g;
	const u32 i = W.regions[r];
	g.dptr = W.dptr[i];
	g.optr = W.optr[i];
	upk(W.pos[i], g.x, g.y, g.z);
	g.unit_levels = P.cfg.L - 1u - C.leaf_level;
	g.units = 1u << (3u * g.unit_levels);
	g.has_src = ctag(g.optr) == kTagLeaf;
	g.fill = fill_of(g.optr);
	if (g.has_src) {
		const u32 *w = C.leaves + cdata(g.optr);
		g.M = w[1];
		g.B = w[2];
		g.W = w[3];
		g.macro = w + 4;
		g.hdr = g.macro + 2u * g.M;
		g.bits = g.hdr + 2u * g.B;
	} else {
		g.M = g.B = g.W = 0;
		g.macro = g.hdr = g.bits = nullptr;
	}
	return g;
}

enum : u32 { kUnitColor = 0, kUnitCopy = 1, kUnitMixed = 2 };

// What unit u of a region becomes: walk the old DAG from the region's node to
// the unit's DAG leaf (VBREditorWrapper::EditNode below leaf_level,
// VBREditor.hpp:61-80).
__device__ __forceinline__ u32 unit_kind(const DevPool &P, const hd_edit_desc &e, const Region &g, u32 u, u64 *leaf,
                                         u32 *lx, u32 *ly, u32 *lz) {
	const u32 L = P.cfg.L, V = L + 1u;
	u32 node = g.dptr, x = g.x, y = g.y, z = g.z;
	for (u32 k = 0; k < g.unit_levels; ++k) {
		const u32 c = (u >> (3u * (g.unit_levels - 1u - k))) & 7u;
		node = dag_child(P, node, c);
		x = (x << 1) | (c & 1u);
		y = (y << 1) | ((c >> 1) & 1u);
		z = (z << 1) | ((c >> 2) & 1u);
		const u32 level = L - g.unit_levels + k; // leaf_level + 1 + k
		const u32 cls = classify(e, V - level, x, y, z);
		if (cls == kClsFull || node == kNull)
			return kUnitColor;
		if (cls == kClsNone)
			return kUnitCopy;
	}
	const u32 *p = node_addr(P, node);
	*leaf = (u64)p[0] | ((u64)p[1] << 32);
	*lx = x;
	*ly = y;
	*lz = z;
	return kUnitMixed;
}

// Old colours of consecutive voxels of a region (VBRChunkIterator, VBRColor.hpp:286-365).
struct SrcCursor {
	u32 blk, end, next_off, wstart;
	__device__ __forceinline__ void start(const Region &g, u32 m) {
		if (!g.has_src)
			return;
		const u32 k = m >> kMacroBits, v = m & (kMacroVoxels - 1u);
		const u32 first = g.macro[2u * k];
		end = k + 1u < g.M ? g.macro[2u * k + 2u] : g.B;
		wstart = g.macro[2u * k + 1u];
		u32 lo = first, hi = end; // last block of the macro whose voxel offset <= v
		while (hi - lo > 1u) {
			const u32 mid = (lo + hi) >> 1;
			if ((g.hdr[2u * mid + 1u] >> 18) <= v)
				lo = mid;
			else
				hi = mid;
		}
		blk = lo;
		next_off = blk + 1u < end ? (g.hdr[2u * (blk + 1u) + 1u] >> 18) : kMacroVoxels;
	}
	__device__ __forceinline__ VCol at(const Region &g, u32 m) {
		if (!g.has_src)
			return g.fill;
		const u32 v = m & (kMacroVoxels - 1u);
		while (v >= next_off) {
			++blk;
			next_off = blk + 1u < end ? (g.hdr[2u * (blk + 1u) + 1u] >> 18) : kMacroVoxels;
		}
		const u32 h1 = g.hdr[2u * blk + 1u], bpw = (h1 >> 16) & 3u;
		u32 wt = 0;
		if (bpw) {
			const u32 bit = wstart + (h1 & 0xFFFFu) + (v - (h1 >> 18)) * bpw, o = bit & 31u;
			wt = g.bits[bit >> 5] >> o;
			if (o + bpw > 32u)
				wt |= g.bits[(bit >> 5) + 1u] << (32u - o);
			wt &= (1u << bpw) - 1u;
		}
		return VCol{g.hdr[2u * blk], wt, bpw, 1u};
	}
};

__device__ __forceinline__ u64 key_of(const VCol &c) { return (u64)c.colors | ((u64)c.bpw << 32); }

// New colour of voxel i of a unit
__device__ __forceinline__ VCol unit_voxel(const hd_edit_desc &e, const EditArgs &a, const Region &g, u32 kind, u64 leaf,
                                           u32 lx, u32 ly, u32 lz, u32 m, u32 i, SrcCursor &src) {
	if (kind == kUnitColor)
		return a.C;
	if (kind == kUnitMixed) {
		const u32 x = (lx << 2) | ((i >> 2) & 2u) | (i & 1u), y = (ly << 2) | ((i >> 3) & 2u) | ((i >> 1) & 1u),
		          z = (lz << 2) | ((i >> 4) & 2u) | ((i >> 2) & 1u);
		if (voxel_in(e, x, y, z) || !((leaf >> i) & 1ull))
			return a.C;
	}
	return src.at(g, m);
}

struct UnitSum {
	u64 first, last;
	u32 heads; // key changes inside the unit
	u32 bits;
};

// A unit that keeps its old colours is the run of old blocks over its 64
// voxels (consecutive blocks of a macro block always differ in colours or bits
// per weight, VBRChunkWriter::append): summarised per block, not per voxel.
__device__ __forceinline__ UnitSum copy_summary(const Region &g, u32 m0) {
	UnitSum s{0, 0, 0, 0};
	if (!g.has_src) {
		s.first = s.last = key_of(g.fill);
		s.bits = 64u * g.fill.bpw;
		return s;
	}
	SrcCursor c;
	c.start(g, m0);
	const u32 v0 = m0 & (kMacroVoxels - 1u), v1 = v0 + 64u;
	u32 v = v0;
	for (;;) {
		const u32 h1 = g.hdr[2u * c.blk + 1u], bpw = (h1 >> 16) & 3u;
		const u64 k = (u64)g.hdr[2u * c.blk] | ((u64)bpw << 32);
		if (v == v0)
			s.first = k;
		s.last = k;
		const u32 stop = c.next_off < v1 ? c.next_off : v1;
		s.bits += (stop - v) * bpw;
		if (c.next_off >= v1)
			break;
		v = c.next_off;
		++s.heads;
		++c.blk;
		c.next_off = c.blk + 1u < c.end ? (g.hdr[2u * (c.blk + 1u) + 1u] >> 18) : kMacroVoxels;
	}
	return s;
}

__device__ __forceinline__ UnitSum unit_summary(const DevPool &P, const EditArgs &a, const Region &g, u32 u) {
	UnitSum s{0, 0, 0, 0};
	u64 leaf = 0;
	u32 lx = 0, ly = 0, lz = 0;
	const u32 kind = unit_kind(P, a.e, g, u, &leaf, &lx, &ly, &lz);
	if (kind == kUnitColor) {
		s.first = s.last = key_of(a.C);
		s.bits = 64u * a.C.bpw;
		return s;
	}
	if (kind == kUnitCopy)
		return copy_summary(g, u * 64u);
	SrcCursor src;
	src.start(g, u * 64u);
	for (u32 i = 0; i < 64u; ++i) {
		const VCol c = unit_voxel(a.e, a, g, kind, leaf, lx, ly, lz, u * 64u + i, i, src);
		const u64 k = key_of(c);
		if (i == 0)
			s.first = k;
		else if (k != s.last)
			++s.heads;
		s.last = k;
		s.bits += c.bpw;
	}
	return s;
}

// Writes one voxel's weight bits at bit position `bit` of the weight words.
__device__ __forceinline__ void put_weight(u32 *wb, u64 bit, u32 weight, u32 bpw) {
	const u32 o = (u32)(bit & 31u);
	atomicOr(&wb[bit >> 5], weight << o);
	if (o + bpw > 32u)
		atomicOr(&wb[(bit >> 5) + 1], weight >> (32u - o));
}

// Headers and weight bits of unit u: block header index hb and bit position
// bb of its first voxel, mws = weight start of its macro block.
__device__ __forceinline__ void emit_unit(const DevPool &P, const EditArgs &a, const Region &g, u32 u, bool head0, u64 hb,
                                          u64 bb, u64 mws, u32 *hdr, u32 *wb) {
	u64 leaf = 0;
	u32 lx = 0, ly = 0, lz = 0;
	const u32 kind = unit_kind(P, a.e, g, u, &leaf, &lx, &ly, &lz);
	const u32 m0 = u * 64u;
	u64 hi = hb, bit = bb;
	auto header = [&](u32 colors, u32 bpw, u32 m) {
		hdr[2ull * hi] = colors;
		hdr[2ull * hi + 1] = ((m & (kMacroVoxels - 1u)) << 18) | (bpw << 16) | (u32)(bit - mws);
		++hi;
	};
	if (kind == kUnitColor || (kind == kUnitCopy && !g.has_src)) {
		const VCol c = kind == kUnitColor ? a.C : g.fill;
		if (head0)
			header(c.colors, c.bpw, m0);
		if (c.bpw)
			for (u32 i = 0; i < 64u; ++i, bit += c.bpw)
				put_weight(wb, bit, c.weight, c.bpw);
		return;
	}
	SrcCursor src;
	src.start(g, m0);
	if (kind == kUnitCopy) { // the old blocks over the unit, their weight bits copied
		const u32 v0 = m0 & (kMacroVoxels - 1u), v1 = v0 + 64u;
		u32 v = v0;
		for (;;) {
			const u32 h0 = g.hdr[2u * src.blk], h1 = g.hdr[2u * src.blk + 1u], bpw = (h1 >> 16) & 3u;
			if (v != v0 || head0)
				header(h0, bpw, (m0 - v0) + v);
			const u32 stop = src.next_off < v1 ? src.next_off : v1;
			if (bpw)
				for (u32 x = v; x < stop; ++x, bit += bpw) {
					const u32 sb = src.wstart + (h1 & 0xFFFFu) + (x - (h1 >> 18)) * bpw, o = sb & 31u;
					u32 w = g.bits[sb >> 5] >> o;
					if (o + bpw > 32u)
						w |= g.bits[(sb >> 5) + 1u] << (32u - o);
					put_weight(wb, bit, w & ((1u << bpw) - 1u), bpw);
				}
			if (src.next_off >= v1)
				break;
			v = src.next_off;
			++src.blk;
			src.next_off = src.blk + 1u < src.end ? (g.hdr[2u * (src.blk + 1u) + 1u] >> 18) : kMacroVoxels;
		}
		return;
	}
	u64 prev = 0;
	for (u32 i = 0; i < 64u; ++i) {
		const u32 m = m0 + i;
		const VCol c = unit_voxel(a.e, a, g, kind, leaf, lx, ly, lz, m, i, src);
		const u64 k = key_of(c);
		if (i == 0 ? head0 : k != prev)
			header(c.colors, c.bpw, m);
		prev = k;
		if (c.bpw) {
			put_weight(wb, bit, c.weight, c.bpw);
			bit += c.bpw;
		}
	}
}

// chunk words (without the block size word) for B blocks and O weight bits
__device__ __forceinline__ u64 chunk_words(u32 M, u64 B, u64 O) { return 3ull + 2ull * M + 2ull * B + (O + 31ull) / 32ull; }

// One CTA per (region, macro block): every macro block starts a VBR block
// (VBRChunkWriter::append), so macro blocks are independent apart from their
// offsets in the chunk.
__global__ void __launch_bounds__(kRegionBlock) k_color_count(DevPool P, ColorDev C, ColorWs W, EditArgs a) {
	__shared__ u64 s_warp[33];
	__shared__ u64 s_last[kRegionBlock];
	const u64 Q = W.c[0] * W.macros;
	for (u64 q = blockIdx.x; q < Q; q += gridDim.x) {
		const u32 r = (u32)(q / W.macros), m = (u32)(q % W.macros);
		const Region g = region_of(P, C, W, r);
		const u32 u = m * kRegionBlock + threadIdx.x;
		UnitSum s{0, 0, 0, 0};
		const bool valid = u < g.units;
		if (valid)
			s = unit_summary(P, a, g, u);
		s_last[threadIdx.x] = s.last;
		__syncthreads();
		u32 h = 0;
		if (valid)
			h = s.heads + ((threadIdx.x == 0 || s.first != s_last[threadIdx.x - 1]) ? 1u : 0u);
		u64 th, tb;
		block_scan(h, s_warp, &th);
		block_scan(s.bits, s_warp, &tb);
		if (threadIdx.x == 0) {
			W.m_blocks[q] = th;
			W.m_bits[q] = tb;
		}
	}
}

// Per region: offsets of its macro blocks' headers and weight bits, the
// chunk's size.
__global__ void __launch_bounds__(kRegionBlock) k_color_region_scan(ColorWs W) {
	__shared__ u64 s_warp[33];
	const u64 R = W.c[0];
	const u32 M = W.macros;
	for (u64 r = blockIdx.x; r < R; r += gridDim.x) {
		u64 B = 0, O = 0;
		for (u32 m0 = 0; m0 < M; m0 += blockDim.x) {
			const u32 m = m0 + threadIdx.x;
			const u64 q = r * M + m;
			const u64 hb = m < M ? W.m_blocks[q] : 0ull, bb = m < M ? W.m_bits[q] : 0ull;
			u64 th, tb;
			const u64 he = block_scan(hb, s_warp, &th), be = block_scan(bb, s_warp, &tb);
			if (m < M) {
				W.m_hoff[q] = B + he;
				W.m_boff[q] = O + be;
			}
			B += th;
			O += tb;
		}
		if (threadIdx.x == 0) {
			W.r_words[r] = (u32)chunk_words(M, B, O);
			W.r_blocks[r] = B;
		}
	}
}

// Scratch offsets and leaf block placement in region order (SetLeaf,
// src/DAGColorPool.hpp:176-207).
__global__ void __launch_bounds__(kWalkBlock) k_color_place(ColorDev C, ColorWs W) {
	__shared__ u64 s_warp[33];
	const u64 R = W.c[0];
	u64 so = 0, app = 0;
	const u64 base = C.ctr[1];
	for (u64 r0 = 0; r0 < R; r0 += blockDim.x) {
		const u64 r = r0 + threadIdx.x;
		u64 words = 0, append = 0, in_place = ~0ull;
		if (r < R) {
			words = W.r_words[r];
			const u64 data_size = words + 1;
			u64 append_size = (data_size & 1) ? data_size + 1 : data_size;
			const u32 o = W.optr[W.regions[r]];
			if (!C.keep_history && ctag(o) == kTagLeaf) {
				const u64 block_size = C.leaves[cdata(o)];
				if (data_size <= block_size)
					in_place = cdata(o);
				else
					append_size = append_size > (block_size << 1) ? append_size : (block_size << 1);
			}
			append = in_place == ~0ull ? append_size : 0;
		}
		u64 ts, ta;
		const u64 s_ex = block_scan(words, s_warp, &ts);
		const u64 a_ex = block_scan(append, s_warp, &ta);
		if (r < R) {
			W.r_scratch[r] = so + s_ex;
			W.r_append[r] = append;
			W.r_dest[r] = append ? base + app + a_ex : in_place;
		}
		so += ts;
		app += ta;
	}
	if (threadIdx.x == 0) {
		W.c[1] = so;
		W.c[2] = app;
		if (so > W.scratch_cap)
			atomicCAS(&W.c[3], 0ull, (unsigned long long)kCErrScratch);
		if (base + app > C.max_leaf_words || base + app > 0x3FFFFFFFull)
			atomicCAS(&W.c[3], 0ull, (unsigned long long)kCErrLeaves);
		// every proceeding node may append one node (checked before any leaf
		// block is rewritten in place)
		const u64 proceed = (W.lvl[C.leaf_level + 1] - 1u) / 8u;
		if (C.ctr[0] + proceed > C.max_nodes || C.ctr[0] + proceed > 0x3FFFFFFFull)
			atomicCAS(&W.c[3], 0ull, (unsigned long long)kCErrNodes);
	}
}

// Scratch of the chunks cleared (weight words are OR-ed in).
__global__ void k_color_zero(ColorWs W) {
	if (W.c[3])
		return;
	const u64 n = W.c[1];
	for (u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (u64)gridDim.x * blockDim.x)
		W.scratch[k] = 0u;
}

// The chunks into scratch (VBRChunkWriter, VBRColor.hpp:367-488), one CTA per
// (region, macro block): unit summaries -> block and bit offsets inside the
// macro block -> headers and weight bits at the macro block's offsets; the
// region's block count places the weight words after the headers.
__global__ void __launch_bounds__(kRegionBlock) k_color_emit(DevPool P, ColorDev C, ColorWs W, EditArgs a) {
	__shared__ u64 s_warp[33];
	__shared__ u64 s_last[kRegionBlock];
	if (W.c[3])
		return;
	const u64 Q = W.c[0] * W.macros;
	for (u64 q = blockIdx.x; q < Q; q += gridDim.x) {
		const u32 r = (u32)(q / W.macros), m = (u32)(q % W.macros), M = W.macros;
		const Region g = region_of(P, C, W, r);
		u32 *out = W.scratch + W.r_scratch[r];
		const u64 btotal = W.r_blocks[r];
		u32 *macro = out + 3, *hdr = macro + 2u * M, *wb = hdr + 2ull * btotal;
		const u64 B = W.m_hoff[q], O = W.m_boff[q];
		const u32 u = m * kRegionBlock + threadIdx.x;
		const bool valid = u < g.units;
		UnitSum s{0, 0, 0, 0};
		if (valid)
			s = unit_summary(P, a, g, u);
		s_last[threadIdx.x] = s.last;
		__syncthreads();
		const bool head0 = valid && (threadIdx.x == 0 || s.first != s_last[threadIdx.x - 1]);
		const u32 h = valid ? s.heads + (head0 ? 1u : 0u) : 0u;
		u64 th, tb;
		const u64 hb = B + block_scan(h, s_warp, &th);
		const u64 bb = O + block_scan(s.bits, s_warp, &tb);
		if (threadIdx.x == 0) {
			macro[2u * m] = (u32)B;
			macro[2u * m + 1u] = (u32)O;
			if (m == 0) {
				out[0] = M;
				out[1] = (u32)btotal;
				out[2] = (u32)((W.m_boff[q + M - 1] + W.m_bits[q + M - 1] + 31u) / 32u);
			}
		}
		if (valid)
			emit_unit(P, a, g, u, head0, hb, bb, O, hdr, wb);
	}
}

__global__ void k_color_copy(ColorDev C, ColorWs W) {
	if (W.c[3])
		return;
	const u64 R = W.c[0];
	for (u64 r = blockIdx.x; r < R; r += gridDim.x) {
		const u64 dest = W.r_dest[r], words = W.r_words[r];
		const u32 *src = W.scratch + W.r_scratch[r];
		for (u64 k = threadIdx.x; k < words; k += blockDim.x)
			C.leaves[dest + 1 + k] = src[k];
		if (threadIdx.x == 0) {
			if (W.r_append[r])
				C.leaves[dest] = (u32)W.r_append[r];
			W.res[W.regions[r]] = cptr(kTagLeaf, (u32)dest);
		}
	}
}

// Morton code of a coordinate at level l (l bits per axis)
__device__ __forceinline__ u64 morton_of(u64 p, u32 l) {
	u32 x, y, z;
	upk(p, x, y, z);
	u64 m = 0;
	for (u32 b = 0; b < l; ++b)
		m |= ((u64)((x >> b) & 1u) << (3 * b)) | ((u64)((y >> b) & 1u) << (3 * b + 1)) |
		     ((u64)((z >> b) & 1u) << (3 * b + 2));
	return m;
}

// SetNode bottom-up (src/DAGColorPool.hpp:150-165) in JoinNode order
// (VBREditor.hpp:92-107): appended nodes are numbered in post order.
__global__ void __launch_bounds__(kWalkBlock) k_color_up(ColorDev C, ColorWs W) {
	__shared__ u64 s_warp[33];
	if (W.c[3])
		return;
	const u32 LL = C.leaf_level;
	// decisions, level LL-1 up to 0
	for (u32 l = LL; l-- > 0;) {
		const u32 b = W.lvl[l], e = W.lvl[l + 1];
		for (u32 i = b + threadIdx.x; i < e; i += blockDim.x) {
			if (W.dec[i] != kDecProceed)
				continue;
			const u32 c0 = W.child[i], o = W.optr[i];
			bool pending = false, all_null = true, same_color = true, stored = ctag(o) == kTagNode;
			const u32 first = W.res[c0];
			for (u32 c = 0; c < 8; ++c) {
				const u32 ch = W.res[c0 + c];
				if (W.app[c0 + c]) {
					pending = true;
					continue;
				}
				all_null = all_null && ctag(ch) == kTagNull;
				same_color = same_color && ch == first;
				stored = stored && C.nodes[(u64)cdata(o) * 8u + c] == ch;
			}
			if (!pending && all_null)
				W.res[i] = kCNull;
			else if (!pending && ctag(first) == kTagColor && same_color)
				W.res[i] = first;
			else if (!pending && stored)
				W.res[i] = o;
			else
				W.app[i] = 1;
		}
		__syncthreads();
	}
	// appended items per level in Morton order, with their end positions
	u64 total = 0;
	for (u32 l = 0; l < LL; ++l) {
		const u32 b = W.lvl[l], e = W.lvl[l + 1];
		if (threadIdx.x == 0)
			W.app_lvl[l] = (u32)total;
		for (u32 i0 = b; i0 < e; i0 += blockDim.x) {
			const u32 i = i0 + threadIdx.x;
			const u32 f = (i < e && W.app[i]) ? 1u : 0u;
			u64 t;
			const u64 ex = block_scan(f, s_warp, &t);
			if (f) {
				const u64 k = total + ex;
				W.app_list[k] = i;
				W.app_end[k] = ((morton_of(W.pos[i], l) + 1ull) << (3u * (LL - l))) - 1ull;
			}
			total += t;
		}
	}
	if (threadIdx.x == 0)
		W.app_lvl[LL] = (u32)total;
	__syncthreads();
	const u64 base = C.ctr[0];
	if (base + total > C.max_nodes || base + total > 0x3FFFFFFFull) {
		if (threadIdx.x == 0)
			atomicCAS(&W.c[3], 0ull, (unsigned long long)kCErrNodes);
		return;
	}
	// rank = appended items before in post order: smaller end, or the same end deeper
	for (u32 l = 0; l < LL; ++l) {
		for (u32 k = W.app_lvl[l] + threadIdx.x; k < W.app_lvl[l + 1]; k += blockDim.x) {
			const u64 end = W.app_end[k];
			u64 rank = 0;
			for (u32 l2 = 0; l2 < LL; ++l2) {
				u32 lo = W.app_lvl[l2], hi = W.app_lvl[l2 + 1];
				// first entry with end >= end (or > end for deeper levels)
				const bool deeper = l2 > l;
				while (lo < hi) {
					const u32 mid = (lo + hi) >> 1;
					const u64 v = W.app_end[mid];
					if (v < end || (deeper && v == end))
						lo = mid + 1;
					else
						hi = mid;
				}
				rank += lo - W.app_lvl[l2];
			}
			const u32 i = W.app_list[k];
			W.nidx[i] = (u32)(base + rank);
			W.res[i] = cptr(kTagNode, (u32)(base + rank));
		}
	}
	__syncthreads();
	for (u64 k = threadIdx.x; k < total; k += blockDim.x) {
		const u32 i = W.app_list[k], c0 = W.child[i];
		for (u32 c = 0; c < 8; ++c)
			C.nodes[(u64)W.nidx[i] * 8u + c] = W.res[c0 + c];
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		W.c[4] = W.res[0];
		W.c[5] = total;
		C.ctr[0] = base + total;
		C.ctr[1] += W.c[2];
	}
}

// trace.frag:303-356 (Color_GetLeafColor / Color_Fetch)
__global__ void k_color_fetch(ColorDev C, u32 voxel_level, u32 root, const u32 *xyz, u32 n, hd_vbr_color *out) {
	const u32 t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n)
		return;
	const u32 v[3] = {xyz[3 * t], xyz[3 * t + 1], xyz[3 * t + 2]};
	u32 p = root;
	for (u32 l = 0; l < C.leaf_level && ctag(p) == kTagNode; ++l) {
		const u32 s = voxel_level - 1u - l;
		p = C.nodes[(u64)cdata(p) * 8u + (((v[0] >> s) & 1u) | (((v[1] >> s) & 1u) << 1) | (((v[2] >> s) & 1u) << 2))];
	}
	VCol c{0, 0, 0, 0};
	if (ctag(p) == kTagColor) {
		c = fill_of(p);
	} else if (ctag(p) == kTagLeaf) {
		c = VCol{0, 0, 0, 1};
		const u32 bits = voxel_level - C.leaf_level;
		u32 vox = 0;
		for (u32 b = 0; b < bits; ++b)
			vox |= (((v[0] >> b) & 1u) << (3 * b)) | (((v[1] >> b) & 1u) << (3 * b + 1)) | (((v[2] >> b) & 1u) << (3 * b + 2));
		const u32 *w = C.leaves + cdata(p);
		const u32 M = w[1], nb = w[2];
		const u32 *macro = w + 4, *hdr = macro + 2u * M, *wb = hdr + 2u * nb;
		const u32 mid = vox >> kMacroBits;
		if (mid < M) {
			const u32 first = macro[2u * mid], wstart = macro[2u * mid + 1u];
			u32 cnt = mid + 1u < M ? macro[2u * mid + 2u] - first : nb - first;
			const u32 *b = hdr + 2u * first;
			vox &= kMacroVoxels - 1u;
			if (cnt) {
				for (u32 it = 0; it <= 14u && cnt != 0u; ++it) {
					const u32 step = cnt >> 1;
					if ((b[2u * step + 1u] >> 18) <= vox) {
						cnt -= step + 1u;
						b += 2u * (step + 1u);
					} else {
						cnt = step;
					}
				}
				b -= 2;
				const u32 bpw = (b[1] >> 16) & 3u;
				c.colors = b[0];
				if (bpw) {
					const u32 bit = wstart + (b[1] & 0xFFFFu) + (vox - (b[1] >> 18)) * bpw, o = bit & 31u;
					u32 wt = wb[bit >> 5] >> o;
					if (o + bpw <= 32u)
						wt &= (1u << bpw) - 1u;
					else
						wt |= (wb[(bit >> 5) + 1u] & ((1u << (o + bpw - 32u)) - 1u)) << (32u - o);
					c.weight = wt;
					c.bpw = bpw;
				}
			}
		}
	}
	float rgb[3];
	vcol_rgb(c, rgb);
	hd_vbr_color r;
	r.has_value = c.has;
	r.colors = c.colors;
	r.weight = c.weight;
	r.bits_per_weight = c.bpw;
	r.rgb[0] = rgb[0];
	r.rgb[1] = rgb[1];
	r.rgb[2] = rgb[2];
	out[t] = r;
}

} // namespace

// ------------------------------------------------------------------ host side
struct hd_color_pool {
	hd_pool *pool = nullptr;
	int device = 0;           // kept here: the colour pool may be destroyed after its node pool
	uint32_t voxel_level = 0;
	uint32_t macros = 1;      // macro blocks per colour leaf
	hd_color_config cfg{};
	ColorDev d{};
	ColorWs w{};
	std::vector<void *> ws_allocs;
	unsigned long long *h_c = nullptr; // pinned copy of the edit counters
	cudaStream_t st = nullptr;
	std::mutex mtx;
};

namespace {

template <typename T> hd_status cp_alloc(hd_color_pool *cp, T **p, uint64_t count) {
	void *q = nullptr;
	if (cudaMalloc(&q, std::max<uint64_t>(count, 1) * sizeof(T)) != cudaSuccess) {
		fprintf(stderr, "hashdag_gb300: colour workspace allocation of %llu bytes failed\n",
		        (unsigned long long)(count * sizeof(T)));
		return HD_ERR_CUDA;
	}
	cp->ws_allocs.push_back(q);
	*p = static_cast<T *>(q);
	return HD_OK;
}

void cp_free_ws(hd_color_pool *cp) {
	for (void *p : cp->ws_allocs)
		cudaFree(p);
	cp->ws_allocs.clear();
	cp->w = ColorWs{};
}

// (Re)allocates the per-edit workspace with at least these capacities.
hd_status cp_reserve(hd_color_pool *cp, uint64_t items, uint64_t regions, uint64_t scratch) {
	ColorWs &w = cp->w;
	if (w.c && w.item_cap >= items && w.region_cap >= regions && w.scratch_cap >= scratch)
		return HD_OK;
	items = std::max<uint64_t>(items, w.item_cap);
	regions = std::max<uint64_t>(regions, w.region_cap);
	scratch = std::max<uint64_t>(scratch, w.scratch_cap);
	HD_TRY(cudaStreamSynchronize(cp->st));
	cp_free_ws(cp);
	ColorWs n{};
	hd_status s;
	if ((s = cp_alloc(cp, &n.pos, items)) || (s = cp_alloc(cp, &n.optr, items)) || (s = cp_alloc(cp, &n.dptr, items)) ||
	    (s = cp_alloc(cp, &n.res, items)) || (s = cp_alloc(cp, &n.dec, items)) || (s = cp_alloc(cp, &n.child, items)) ||
	    (s = cp_alloc(cp, &n.app, items)) || (s = cp_alloc(cp, &n.nidx, items)) ||
	    (s = cp_alloc(cp, &n.lvl, (uint64_t)HD_MAX_LEVELS + 2)) || (s = cp_alloc(cp, &n.regions, regions)) ||
	    (s = cp_alloc(cp, &n.r_words, regions)) || (s = cp_alloc(cp, &n.r_blocks, regions)) ||
	    (s = cp_alloc(cp, &n.r_scratch, regions)) || (s = cp_alloc(cp, &n.r_dest, regions)) ||
	    (s = cp_alloc(cp, &n.r_append, regions)) || (s = cp_alloc(cp, &n.scratch, scratch)) ||
	    (s = cp_alloc(cp, &n.app_list, items)) || (s = cp_alloc(cp, &n.app_lvl, (uint64_t)HD_MAX_LEVELS + 2)) ||
	    (s = cp_alloc(cp, &n.app_end, items)) || (s = cp_alloc(cp, &n.c, 8)) ||
	    (s = cp_alloc(cp, &n.m_blocks, regions * cp->macros)) || (s = cp_alloc(cp, &n.m_bits, regions * cp->macros)) ||
	    (s = cp_alloc(cp, &n.m_hoff, regions * cp->macros)) || (s = cp_alloc(cp, &n.m_boff, regions * cp->macros))) {
		cp_free_ws(cp);
		return s;
	}
	n.macros = cp->macros;
	n.item_cap = items;
	n.region_cap = regions;
	n.scratch_cap = scratch;
	w = n;
	return HD_OK;
}

uint64_t isqrt_u64(uint64_t v) {
	uint64_t r = (uint64_t)std::sqrt((double)v);
	while (r * r > v)
		--r;
	while ((r + 1) * (r + 1) <= v)
		++r;
	return r;
}

// Walk items and regions an edit can produce: a node proceeds only where the
// edit's bounding box overlaps it, and each proceeding node has 8 children.
// The sphere classification (src/main.cpp:77-106) measures distances to a
// node's exclusive upper bound, so a sphere also "touches" the nodes that end
// one voxel before it: its box is widened by one voxel on each side.
void walk_bounds(const hd_edit_desc &e, uint32_t voxel_level, uint32_t leaf_level, uint64_t *items, uint64_t *regions) {
	const uint64_t res = 1ull << voxel_level;
	int64_t lo[3], hi[3];
	for (int a = 0; a < 3; ++a) {
		if (e.shape == HD_SHAPE_AABB) {
			lo[a] = e.p0[a];
			hi[a] = e.p1[a];
		} else {
			const int64_t r = (int64_t)isqrt_u64(e.r2);
			lo[a] = (int64_t)e.p0[a] - r - 1;
			hi[a] = (int64_t)e.p0[a] + r + 2;
		}
		lo[a] = std::max<int64_t>(lo[a], 0);
		hi[a] = std::min<int64_t>(hi[a], (int64_t)res);
	}
	uint64_t total = 1, at = 1; // items at the current level
	for (uint32_t l = 0; l <= leaf_level; ++l) {
		uint64_t cells = 1;
		for (int a = 0; a < 3; ++a) {
			const uint32_t s = voxel_level - l;
			cells *= hi[a] > lo[a] ? (uint64_t)(((hi[a] - 1) >> s) - (lo[a] >> s) + 1) : 0ull;
		}
		const uint64_t proceed = std::min(cells, at);
		if (l == leaf_level) {
			*regions = std::max<uint64_t>(proceed, 1);
			break;
		}
		at = 8 * proceed;
		total += at;
	}
	*items = total + 8;
}

hd_status cp_check(cudaError_t e) { return e == cudaSuccess ? HD_OK : HD_ERR_CUDA; }

} // namespace

extern "C" {

hd_status hd_color_pool_create(hd_pool *pool, const hd_color_config *cfg, hd_color_pool **out) {
	if (!pool || !cfg || !out)
		return HD_ERR_INVALID_ARG;
	*out = nullptr;
	const uint32_t L = pool->cfg.node_levels, V = L + 1;
	// a colour leaf holds at most 2^24 voxels and lies at or above the DAG's leaf level
	if (cfg->leaf_level + 1 > L || V - cfg->leaf_level > 8 || cfg->max_nodes == 0 || cfg->max_leaf_words == 0 ||
	    cfg->max_nodes > (1ull << 30) || cfg->max_leaf_words > (1ull << 30))
		return HD_ERR_INVALID_ARG;
	auto *cp = new hd_color_pool;
	cp->pool = pool;
	cp->device = pool->device;
	cp->voxel_level = V;
	cp->macros = std::max<uint32_t>(1u, (uint32_t)((1ull << (3u * (V - cfg->leaf_level))) >> kMacroBits));
	cp->cfg = *cfg;
	if (cudaSetDevice(pool->device) != cudaSuccess) {
		delete cp;
		return HD_ERR_CUDA;
	}
	ColorDev &d = cp->d;
	d.max_nodes = cfg->max_nodes;
	d.max_leaf_words = cfg->max_leaf_words;
	d.leaf_level = cfg->leaf_level;
	d.keep_history = cfg->keep_history ? 1u : 0u;
	if (cudaMalloc(&d.nodes, cfg->max_nodes * 32ull) != cudaSuccess ||
	    cudaMalloc(&d.leaves, cfg->max_leaf_words * 4ull) != cudaSuccess ||
	    cudaMalloc(&d.ctr, 4 * sizeof(unsigned long long)) != cudaSuccess ||
	    cudaMallocHost(&cp->h_c, 8 * sizeof(unsigned long long)) != cudaSuccess ||
	    cudaStreamCreateWithFlags(&cp->st, cudaStreamNonBlocking) != cudaSuccess) {
		hd_color_pool_destroy(cp);
		return HD_ERR_CUDA;
	}
	// appended leaf blocks read as zero past their data, like freshly appended words
	if (cudaMemsetAsync(d.leaves, 0, cfg->max_leaf_words * 4ull, cp->st) != cudaSuccess ||
	    cudaMemsetAsync(d.ctr, 0, 4 * sizeof(unsigned long long), cp->st) != cudaSuccess ||
	    cudaStreamSynchronize(cp->st) != cudaSuccess) {
		hd_color_pool_destroy(cp);
		return HD_ERR_CUDA;
	}
	*out = cp;
	return HD_OK;
}

void hd_color_pool_destroy(hd_color_pool *cp) {
	if (!cp)
		return;
	cudaSetDevice(cp->device);
	if (cp->st)
		cudaStreamSynchronize(cp->st);
	cp_free_ws(cp);
	cudaFree(cp->d.nodes);
	cudaFree(cp->d.leaves);
	cudaFree(cp->d.ctr);
	if (cp->h_c)
		cudaFreeHost(cp->h_c);
	if (cp->st)
		cudaStreamDestroy(cp->st);
	delete cp;
}

hd_status hd_color_pool_read(hd_color_pool *cp, uint32_t *nodes, uint64_t *n_nodes, uint32_t *leaves,
                             uint64_t *n_leaf_words) {
	if (!cp || !n_nodes || !n_leaf_words)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(cp->mtx);
	HD_TRY(cudaSetDevice(cp->device));
	unsigned long long c[2];
	HD_TRY(cudaMemcpyAsync(c, cp->d.ctr, sizeof(c), cudaMemcpyDeviceToHost, cp->st));
	HD_TRY(cudaStreamSynchronize(cp->st));
	*n_nodes = c[0];
	*n_leaf_words = c[1];
	if (nodes && c[0])
		HD_TRY(cudaMemcpyAsync(nodes, cp->d.nodes, c[0] * 32ull, cudaMemcpyDeviceToHost, cp->st));
	if (leaves && c[1])
		HD_TRY(cudaMemcpyAsync(leaves, cp->d.leaves, c[1] * 4ull, cudaMemcpyDeviceToHost, cp->st));
	HD_TRY(cudaStreamSynchronize(cp->st));
	return HD_OK;
}

hd_status hd_vbr_edit(hd_pool *pool, hd_color_pool *cp, uint32_t root, uint32_t color_root, const hd_vbr_edit_desc *edits,
                      uint32_t n, uint32_t *out_root, uint32_t *out_color_root) {
	if (!pool || !cp || cp->pool != pool || !out_root || !out_color_root || (n && !edits))
		return HD_ERR_INVALID_ARG;
	for (uint32_t i = 0; i < n; ++i) {
		const hd_vbr_edit_desc &v = edits[i];
		if (v.edit.shape > HD_SHAPE_AABB || v.edit.op > HD_OP_PAINT || v.bits_per_weight > 3 ||
		    (v.bits_per_weight == 0 ? v.weight != 0 : v.weight >= (1u << v.bits_per_weight)))
			return HD_ERR_INVALID_ARG;
	}
	*out_root = root;
	*out_color_root = color_root;
	const uint32_t L = pool->cfg.node_levels, V = L + 1;
	const uint64_t sms = (uint64_t)pool->num_sms;
	for (uint32_t i = 0; i < n; ++i) {
		const hd_vbr_edit_desc &v = edits[i];
		const bool colour = v.edit.op != HD_OP_DIG;
		hd_edit_desc g = v.edit;
		g.op = HD_OP_FILL;
		EditArgs a{};
		uint64_t items = 0, regions = 0;
		if (colour) {
			a.e = g;
			// VBRColor(RGB8Color) keeps 24 bits (Color.hpp:21)
			a.C = VCol{v.bits_per_weight ? v.colors : (v.colors & 0xFFFFFFu), v.weight, v.bits_per_weight, 1u};
			a.rgb8 = vcol_rgb8(a.C);
			a.root = root;
			a.color_root = color_root;
			walk_bounds(g, V, cp->cfg.leaf_level, &items, &regions);
		}
		// one edit at a time per colour pool (its workspace and pinned counters);
		// lock order: colour pool, then node pool (hd_edit takes the latter)
		std::lock_guard<std::mutex> lk_cp(cp->mtx);
		// the colour part of the edit, against the DAG before the edit; it
		// overlaps the geometry pass (which only adds nodes) and reports
		// errors on the device, read after both
		auto launch_colour = [&]() -> hd_status {
			std::lock_guard<std::mutex> lk(pool->mtx);
			HD_TRY(cudaSetDevice(pool->device));
			hd_status s = cp_reserve(cp, items, regions, cp->w.scratch_cap ? cp->w.scratch_cap : (1ull << 22));
			if (s)
				return s;
			const ColorWs &w = cp->w;
			cudaStream_t st = cp->st;
			const uint64_t q = regions * cp->macros;
			const uint32_t gq = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(q, sms * 8));
			const uint32_t gr = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(regions, sms * 2));
			HD_TRY(cudaStreamWaitEvent(st, pool->ws_free, 0)); // passes of the DAG pool that wrote nodes
			HD_TRY(cudaMemsetAsync(w.c, 0, 8 * sizeof(unsigned long long), st));
			k_color_walk<<<1, kWalkBlock, 0, st>>>(pool->P, cp->d, w, a);
			k_color_count<<<gq, kRegionBlock, 0, st>>>(pool->P, cp->d, w, a);
			k_color_region_scan<<<gr, kRegionBlock, 0, st>>>(w);
			k_color_place<<<1, kWalkBlock, 0, st>>>(cp->d, w);
			k_color_zero<<<(uint32_t)(sms * 4), 256, 0, st>>>(w);
			k_color_emit<<<gq, kRegionBlock, 0, st>>>(pool->P, cp->d, w, a);
			k_color_copy<<<gr, 256, 0, st>>>(cp->d, w);
			k_color_up<<<1, kWalkBlock, 0, st>>>(cp->d, w);
			pool->kernel_launches += 8;
			HD_TRY(cudaGetLastError());
			HD_TRY(cudaMemcpyAsync(cp->h_c, w.c, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
			return HD_OK;
		};
		if (colour) {
			hd_status s = launch_colour();
			if (s)
				return s;
		}
		uint32_t new_root = root;
		if (v.edit.op != HD_OP_PAINT) { // geometry: a fill, or a stateless dig
			hd_edit_desc ge = v.edit;
			hd_status s = hd_edit(pool, root, &ge, 1, &new_root, nullptr);
			if (s)
				return s;
		}
		if (colour) {
			for (int attempt = 0;; ++attempt) {
				HD_TRY(cudaStreamSynchronize(cp->st));
				const unsigned long long err = cp->h_c[3];
				if (err == kCErrScratch && attempt == 0) { // more scratch, then the colour part again
					const uint64_t need = cp->h_c[1];
					{
						HD_TRY(cudaSetDevice(pool->device));
						hd_status s = cp_reserve(cp, items, regions, need);
						if (s)
							return s;
					}
					hd_status s = launch_colour();
					if (s)
						return s;
					continue;
				}
				if (err == kCErrNodes || err == kCErrLeaves)
					return HD_ERR_POOL_OOM; // this edit not applied: both roots stay
				if (err) { // the walk bounds are upper bounds: a capacity error is a bug
					fprintf(stderr,
					        "hashdag_gb300: hd_vbr_edit: colour edit %u failed (code %llu: regions %llu, scratch words "
					        "%llu, item bound %llu, region bound %llu)\n",
					        i, err, cp->h_c[0], cp->h_c[1], (unsigned long long)items, (unsigned long long)regions);
					return HD_ERR_INTERNAL;
				}
				break;
			}
			color_root = (uint32_t)cp->h_c[4];
		}
		root = new_root;
		*out_root = root;
		*out_color_root = color_root;
	}
	return HD_OK;
}

hd_status hd_color_fetch(hd_color_pool *cp, uint32_t color_root, const uint32_t *d_xyz, uint32_t n,
                         hd_vbr_color *d_out, void *stream) {
	if (!cp || (n && (!d_xyz || !d_out)))
		return HD_ERR_INVALID_ARG;
	if (n == 0)
		return HD_OK;
	HD_TRY(cudaSetDevice(cp->device));
	cudaStream_t st = (cudaStream_t)stream;
	k_color_fetch<<<(n + 255) / 256, 256, 0, st>>>(cp->d, cp->voxel_level, color_root, d_xyz, n, d_out);
	return cp_check(cudaGetLastError());
}

} // extern "C"
