// hd_trace.cu -- read path: DAG ray traversal and point queries.
//
// k_trace restates NodePoolTraversal::Traversal<float>
// (include/hashdag/NodePoolTraversal.hpp:93-256), the Laine-Karras style
// traversal of the DAG mapped to [1,2]^3, with the voxel position / size
// output of shader/src/trace.frag:223-246 and without the LOD cut.  One thread
// per ray; this file is compiled with -fmad=false and IEEE division / square
// root so every float operation rounds exactly like the CPU restatement built
// with -ffp-contract=off.
#include "hd_internal.h"

#include <cmath>

#include <algorithm>
#include <cstdio>

using namespace hd;

namespace {

constexpr uint32_t kBeamBlock = 8; // src/rg/BeamPass.cpp:11 kBlockSize

__device__ __forceinline__ float fmin_ref(float x, float y) { return (y < x) ? y : x; } // glm::min
__device__ __forceinline__ float fmax_ref(float x, float y) { return (x < y) ? y : x; } // glm::max
__device__ __forceinline__ float abs_ref(float x) { return x >= 0.0f ? x : -x; }

// Stackless form of the traversal's parent stack.  The reference keeps one
// node per scale (23 entries per ray) and pops by reading it back.  Here a ray
// keeps only the nodes of its last four pushed scales in registers (a ring
// indexed by scale & 3, with each entry's scale in one byte of `sc`); a pop
// to a scale the ring no longer holds re-descends from the root along the
// position bits of the ray's current cell, which name the child taken at
// every scale, so it arrives at the very node the reference's stack holds.
// Only node pointers come from the stack (no t value is restored on a pop),
// so every float operation of the traversal, and its result, is unchanged.
struct ParentRing {
	u32 n0, n1, n2, n3;
	u32 sc = 0xFFFFFFFFu; // byte k: scale of entry k, 0xFF = empty
	__device__ __forceinline__ void push(int scale, u32 node) {
		const u32 k = (u32)scale & 3u;
		n0 = k == 0u ? node : n0;
		n1 = k == 1u ? node : n1;
		n2 = k == 2u ? node : n2;
		n3 = k == 3u ? node : n3;
		sc = (sc & ~(0xFFu << (8u * k))) | ((u32)scale << (8u * k));
	}
	// The node of `scale` if the ring holds it; kNull otherwise.  Entries of
	// lower scales belong to the subtree being left and are dropped.
	__device__ __forceinline__ u32 pop(int scale) {
		const u32 k = (u32)scale & 3u;
		const bool have = ((sc >> (8u * k)) & 0xFFu) == (u32)scale;
		const u32 node = k == 0u ? n0 : (k == 1u ? n1 : (k == 2u ? n2 : n3));
		sc |= __vcmpltu4(sc, 0x01010101u * (u32)scale); // bytes below `scale` -> 0xFF
		return have ? node : kNull;
	}
};
// The node at `scale` on the path of the cell at pos (scale > leaf scale):
// from the root, each scale's child index is that scale's position bit per
// axis, mirrored by the octant (as in the descent).
__device__ __forceinline__ u32 descend_to(const DevPool &P, u32 root, int top, int scale, const float pos[3], u32 octant,
                                          u32 *reads) {
	u32 node = root;
	for (int sc = top; sc > scale; --sc) {
		const u32 idx = ((__float_as_uint(pos[0]) >> sc) & 1u) | (((__float_as_uint(pos[1]) >> sc) & 1u) << 1) |
		                (((__float_as_uint(pos[2]) >> sc) & 1u) << 2);
		const u32 cs = idx ^ octant;
		const u32 *p = node_addr(P, node);
		node = node_addr(P, node + 1u + __popc(p[0] & ((1u << cs) - 1u)))[0];
		*reads += 2;
	}
	return node;
}

// One ray of the traversal as a state machine: init() is the prologue, each
// step() one iteration of the reference's loop (true once the ray is done),
// finish() the hit record.  trace_core runs them back to back; the persistent
// kernel below interleaves rays on a lane.  The float operations are the
// reference's, in its order, whichever way the steps are scheduled.
// steps: loop iterations; reads: node words fetched (mask words, child pointers, leaf words).
// Lod: the level-of-detail cut of shader/src/trace.frag:148 and beam.frag:128 --
// descent stops at a cube whose size times proj_factor is below its entry t plus
// proj_bias; finish() reports the size of the cube the ray stopped in.
// Stackless: the parent stack is a ParentRing plus re-descents (same result).
constexpr int kStack = 23;
// The stackful form keeps its parent stack outside the struct (a local array
// of the caller, passed to init and step), so the rest of the state stays in
// registers.
template <bool Lod, bool Stackless> struct Ray {
	ParentRing ring;
	float o[3], d[3], tc[3], tb[3];
	float t_min, t_max, h, scale_exp2, pos[3];
	float proj_factor, proj_bias;
	u32 octant, parent, child_bits, idx, n_steps, n_reads;
	int scale;

	__device__ __forceinline__ void init(u32 root, float ox, float oy, float oz, float dx, float dy, float dz,
	                                     float pf, float pb, u32 *stack) {
		const float eps = __uint_as_float((127u - 23u) << 23);
		n_steps = n_reads = 0;
		proj_factor = pf;
		proj_bias = pb;
		ring = ParentRing{};
		if (!Stackless) {
#pragma unroll
			for (int k = 0; k < kStack; ++k) // every entry holds a node pointer before the first push
				stack[k] = root;
		}
		o[0] = ox + 1.0f;
		o[1] = oy + 1.0f;
		o[2] = oz + 1.0f;
		const float din[3] = {dx, dy, dz};
#pragma unroll
		for (int a = 0; a < 3; ++a)
			d[a] = abs_ref(din[a]) > eps ? din[a] : (din[a] >= 0.0f ? eps : -eps);
#pragma unroll
		for (int a = 0; a < 3; ++a) {
			tc[a] = __fdiv_rn(1.0f, -abs_ref(d[a]));
			tb[a] = __fmul_rn(tc[a], o[a]);
		}
		octant = 0;
#pragma unroll
		for (int a = 0; a < 3; ++a)
			if (d[a] > 0.0f) {
				octant ^= 1u << a;
				tb[a] = __fsub_rn(__fmul_rn(3.0f, tc[a]), tb[a]);
			}
		t_min = fmax_ref(fmax_ref(__fsub_rn(__fmul_rn(2.0f, tc[0]), tb[0]), __fsub_rn(__fmul_rn(2.0f, tc[1]), tb[1])),
		                 __fsub_rn(__fmul_rn(2.0f, tc[2]), tb[2]));
		t_max = fmin_ref(fmin_ref(__fsub_rn(tc[0], tb[0]), __fsub_rn(tc[1], tb[1])), __fsub_rn(tc[2], tb[2]));
		h = t_max;
		t_min = fmax_ref(t_min, 0.0f);
		t_max = fmin_ref(t_max, 1.0f);
		parent = root;
		child_bits = 0;
		pos[0] = pos[1] = pos[2] = 1.0f;
		idx = 0;
#pragma unroll
		for (int a = 0; a < 3; ++a)
			if (__fsub_rn(__fmul_rn(1.5f, tc[a]), tb[a]) > t_min) {
				idx ^= 1u << a;
				pos[a] = 1.5f;
			}
		scale = kStack - 1;
		scale_exp2 = 0.5f;
	}

	// One loop iteration (NodePoolTraversal.hpp:151-243); true when the ray stops
	// (a hit below the leaf scale or at the level-of-detail cut, or it leaves the
	// root), in which case the state is the one the reference's loop breaks with.
	__device__ __forceinline__ bool step(const DevPool &P, u32 root, int leaf_scale, u32 *stack) {
		++n_steps;
		if (child_bits == 0u) {
			if (scale > leaf_scale) {
				child_bits = node_addr(P, parent)[0];
				++n_reads;
			} else if (scale == leaf_scale) {
				n_reads += 2;
				const u32 *p = node_addr(P, parent);
				const u32 l0 = p[0], l1 = p[1];
				child_bits = ((l0 & 0xFFu) ? 1u : 0u) | ((l0 & 0xFF00u) ? 2u : 0u) | ((l0 & 0xFF0000u) ? 4u : 0u) |
				             ((l0 & 0xFF000000u) ? 8u : 0u) | ((l1 & 0xFFu) ? 16u : 0u) | ((l1 & 0xFF00u) ? 32u : 0u) |
				             ((l1 & 0xFF0000u) ? 64u : 0u) | ((l1 & 0xFF000000u) ? 128u : 0u);
			} else
				child_bits = parent;
		}
		float tcor[3];
#pragma unroll
		for (int a = 0; a < 3; ++a)
			tcor[a] = __fsub_rn(__fmul_rn(pos[a], tc[a]), tb[a]);
		const float tc_max = fmin_ref(fmin_ref(tcor[0], tcor[1]), tcor[2]);
		const u32 child_shift = idx ^ octant;
		const u32 child_mask = 1u << child_shift;
		if ((child_bits & child_mask) != 0 && t_min <= t_max) {
			const float half = __fmul_rn(scale_exp2, 0.5f);
			float tcen[3];
#pragma unroll
			for (int a = 0; a < 3; ++a)
				tcen[a] = __fadd_rn(__fmul_rn(half, tc[a]), tcor[a]);
			if (scale < leaf_scale || (Lod && __fmul_rn(scale_exp2, proj_factor) < __fadd_rn(tc_max, proj_bias)))
				return true;
			if (tc_max < h) {
				if (Stackless)
					ring.push(scale, parent);
				else
					stack[scale] = parent;
			}
			h = tc_max;
			if (scale > leaf_scale)
				parent = node_addr(P, parent + 1u + __popc(child_bits & (child_mask - 1u)))[0];
			else
				parent = (node_addr(P, parent + (child_shift >> 2u))[0] >> ((child_shift & 3u) << 3u)) & 0xFFu;
			++n_reads;
			idx = 0;
			--scale;
			scale_exp2 = half;
#pragma unroll
			for (int a = 0; a < 3; ++a)
				if (tcen[a] > t_min) {
					idx ^= 1u << a;
					pos[a] = __fadd_rn(pos[a], scale_exp2);
				}
			child_bits = 0;
			return false;
		}
		u32 stp = 0;
#pragma unroll
		for (int a = 0; a < 3; ++a)
			if (tcor[a] <= tc_max) {
				stp ^= 1u << a;
				pos[a] = __fsub_rn(pos[a], scale_exp2);
			}
		t_min = tc_max;
		idx ^= stp;
		if ((idx & stp) != 0) {
			u32 diff = 0;
#pragma unroll
			for (int a = 0; a < 3; ++a)
				if (stp & (1u << a))
					diff |= __float_as_uint(pos[a]) ^ __float_as_uint(__fadd_rn(pos[a], scale_exp2));
			scale = diff ? 31 - __clz(diff) : -1;
			if (scale >= kStack || scale < 0) {
				scale = kStack;
				return true;
			}
			scale_exp2 = __uint_as_float((u32)(scale - kStack + 127) << 23);
			u32 sh[3];
#pragma unroll
			for (int a = 0; a < 3; ++a) {
				sh[a] = __float_as_uint(pos[a]) >> scale;
				pos[a] = __uint_as_float(sh[a] << scale);
			}
			if (Stackless) {
				parent = ring.pop(scale);
				if (parent == kNull)
					parent = descend_to(P, root, kStack - 1, scale, pos, octant, &n_reads);
			} else {
				parent = stack[scale];
			}
			idx = (sh[0] & 1u) | ((sh[1] & 1u) << 1) | ((sh[2] & 1u) << 2);
			h = 0.0f;
			child_bits = 0;
		}
		return false;
	}

	// The hit record of a stopped ray (trace.frag:223-246 for the voxel output).
	__device__ __forceinline__ hd_hit finish(u32 leaf_level) const {
		hd_hit out;
		out.voxel[0] = out.voxel[1] = out.voxel[2] = 0;
		out.size = 0;
		out.level = 0;
		const bool hit = scale < kStack && t_min <= t_max;
		out.hit = hit ? 1u : 0u;
		out.t = t_min;
		out.pos[0] = out.pos[1] = out.pos[2] = 0.0f;
		const u32 voxel_level = leaf_level + 1u;
		const int voxel_scale = kStack - (int)voxel_level;
		if (hit) {
			const u32 size = 1u << (scale - voxel_scale);
#pragma unroll
			for (int a = 0; a < 3; ++a) {
				u32 vp = (__float_as_uint(pos[a]) & 0x7FFFFFu) >> voxel_scale;
				if (octant & (1u << a))
					vp = (1u << voxel_level) - size - vp;
				out.voxel[a] = vp;
			}
			out.size = size;
			out.level = voxel_level - (31u - __clz(size));
#pragma unroll
			for (int a = 0; a < 3; ++a) {
				float p = pos[a];
				if (octant & (1u << a))
					p = __fsub_rn(__fsub_rn(3.0f, scale_exp2), p);
				float q = __fadd_rn(o[a], __fmul_rn(t_min, d[a]));
				q = fmin_ref(fmax_ref(q, p), __fadd_rn(p, scale_exp2));
				out.pos[a] = __fsub_rn(q, 1.0f);
			}
		}
		return out;
	}
};

// A ray that runs past this many loop iterations stops (a ray crosses at most
// a few thousand cells).
constexpr u32 kRaySteps = 1u << 20;

template <bool Lod, bool Stackless = false>
__device__ hd_hit trace_core(const DevPool &P, u32 root, float ox, float oy, float oz, float dx, float dy, float dz,
                             float proj_factor, float proj_bias, u32 *steps, u32 *reads, float *scale_out) {
	if (root == kNull) {
		hd_hit out;
		out.voxel[0] = out.voxel[1] = out.voxel[2] = 0;
		out.size = out.level = out.hit = 0;
		out.t = 0.0f;
		out.pos[0] = out.pos[1] = out.pos[2] = 0.0f;
		if (steps)
			*steps = 0;
		if (reads)
			*reads = 0;
		return out;
	}
	Ray<Lod, Stackless> r;
	u32 stack[Stackless ? 1 : kStack];
	r.init(root, ox, oy, oz, dx, dy, dz, proj_factor, proj_bias, stack);
	const int leaf_scale = kStack - (int)P.cfg.L;
	while (r.n_steps < kRaySteps && !r.step(P, root, leaf_scale, stack)) {
	}
	if (steps)
		*steps = r.n_steps;
	if (reads)
		*reads = r.n_reads;
	if (scale_out)
		*scale_out = r.scale_exp2;
	return r.finish(P.cfg.L);
}

__device__ __forceinline__ hd_hit trace_one(const DevPool &P, u32 root, float ox, float oy, float oz, float dx,
                                            float dy, float dz, u32 *steps = nullptr, u32 *reads = nullptr) {
	return trace_core<false>(P, root, ox, oy, oz, dx, dy, dz, 0.0f, 0.0f, steps, reads, nullptr);
}

// Camera_GenRay (shader/src/trace.frag:366-370) at the centre of pixel (px, py)
// of a w x h image, normalised with the same float operations as the host.
__device__ __forceinline__ void pinhole_dir(const hd_camera &cam, u32 px, u32 py, u32 w, u32 h, float d[3]) {
	const float u = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn((float)px, 0.5f), (float)w), 2.0f), 1.0f);
	const float v = __fsub_rn(__fmul_rn(__fdiv_rn(__fadd_rn((float)py, 0.5f), (float)h), 2.0f), 1.0f);
	float dd[3];
#pragma unroll
	for (int a = 0; a < 3; ++a)
		dd[a] = __fsub_rn(__fsub_rn(cam.look[a], __fmul_rn(cam.side[a], u)), __fmul_rn(cam.up[a], v));
	const float len2 = __fadd_rn(__fadd_rn(__fmul_rn(dd[0], dd[0]), __fmul_rn(dd[1], dd[1])), __fmul_rn(dd[2], dd[2]));
	const float inv = __fdiv_rn(1.0f, __fsqrt_rn(len2));
#pragma unroll
	for (int a = 0; a < 3; ++a)
		d[a] = __fmul_rn(dd[a], inv);
}

__device__ __forceinline__ void warp_add_counters(unsigned long long *counters, u64 a, u64 b, u64 c) {
	for (int k = 16; k > 0; k >>= 1) {
		a += __shfl_down_sync(0xFFFFFFFFu, a, k);
		b += __shfl_down_sync(0xFFFFFFFFu, b, k);
		c += __shfl_down_sync(0xFFFFFFFFu, c, k);
	}
	if ((threadIdx.x & 31u) == 0) {
		atomicAdd(counters + 0, (unsigned long long)a);
		atomicAdd(counters + 1, (unsigned long long)b);
		atomicAdd(counters + 2, (unsigned long long)c);
	}
}

// beam.frag main: one ray per block of the beam image (bw x bh per camera),
// t = max(t_hit - size of the stopping cube, 0), +inf where the ray misses.
__global__ void k_beam(DevPool P, u32 root, const hd_camera *cams, u32 n_cams, u32 bw, u32 bh, float proj_factor,
                       float *beam, unsigned long long *counters) {
	const u64 per = (u64)bw * bh, total = per * n_cams;
	u64 my_steps = 0, my_reads = 0;
	for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x) {
		const u32 c = (u32)(i / per);
		const u32 px = (u32)(i % per % bw), py = (u32)(i % per / bw);
		const hd_camera cam = cams[c];
		float d[3];
		pinhole_dir(cam, px, py, bw, bh, d);
		u32 st_, rd_;
		float sexp = 0.0f;
		const hd_hit hh = trace_core<true>(P, root, cam.position[0], cam.position[1], cam.position[2], d[0], d[1], d[2],
		                                   proj_factor, 0.0f, &st_, &rd_, &sexp);
		beam[i] = hh.hit ? fmax_ref(__fsub_rn(hh.t, sexp), 0.0f) : __uint_as_float(0x7F800000u);
		my_steps += st_;
		my_reads += rd_;
	}
	if (counters)
		warp_add_counters(counters, my_steps, my_reads, 0);
}

// Beam value of pixel (px, py): textureLod(uBeam, coord, 0) with a linear
// sampler in MIN reduction mode and clamp-to-edge (src/rg/TracePass.cpp:37-54),
// i.e. the minimum of the 2x2 texels around x = coord * size - 0.5, the
// footprint taken with exact rational arithmetic; times 0.98 (trace.frag:385).
__device__ __forceinline__ int floor_div(long long a, long long b) {
	return (int)(a >= 0 ? a / b : -((-a + b - 1) / b));
}
__device__ __forceinline__ float beam_at(const float *beam, u32 px, u32 py, u32 w, u32 h, u32 bw, u32 bh) {
	const int i0 = floor_div((2ll * px + 1) * bw - w, 2ll * w), j0 = floor_div((2ll * py + 1) * bh - h, 2ll * h);
	const int xs[2] = {max(0, min(i0, (int)bw - 1)), max(0, min(i0 + 1, (int)bw - 1))};
	const int ys[2] = {max(0, min(j0, (int)bh - 1)), max(0, min(j0 + 1, (int)bh - 1))};
	float m = beam[(u64)ys[0] * bw + xs[0]];
#pragma unroll
	for (int k = 1; k < 4; ++k)
		m = fmin_ref(m, beam[(u64)ys[k >> 1] * bw + xs[k & 1]]);
	return __fmul_rn(m, 0.98f);
}

// trace.frag main with BEAM_OPTIMIZATION (beam != nullptr) or without it:
// the level-of-detail traversal from the camera, or from o + beam * d with the
// beam value as projection bias.
__global__ void k_trace_pinhole_lod(DevPool P, u32 root, const hd_camera *cams, u32 n_cams, u32 w, u32 h,
                                    float proj_factor, const float *beam, u32 bw, u32 bh, hd_hit *out,
                                    unsigned long long *counters) {
	const u64 per = (u64)w * h, total = per * n_cams;
	u64 my_steps = 0, my_reads = 0, my_hits = 0;
	for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x) {
		const u32 c = (u32)(i / per);
		const u32 px = (u32)(i % per % w), py = (u32)(i % per / w);
		const hd_camera cam = cams[c];
		float d[3], o[3] = {cam.position[0], cam.position[1], cam.position[2]};
		pinhole_dir(cam, px, py, w, h, d);
		float bias = 0.0f;
		bool traced = true;
		if (beam) {
			bias = beam_at(beam + (u64)c * bw * bh, px, py, w, h, bw, bh);
			traced = __float_as_uint(bias) != 0x7F800000u; // isinf: the block's ray missed
#pragma unroll
			for (int a = 0; a < 3; ++a)
				o[a] = __fadd_rn(o[a], __fmul_rn(bias, d[a]));
		}
		hd_hit hh{};
		u32 st_ = 0, rd_ = 0;
		if (traced)
			hh = trace_core<true>(P, root, o[0], o[1], o[2], d[0], d[1], d[2], proj_factor, bias, &st_, &rd_, nullptr);
		out[i] = hh;
		my_steps += st_;
		my_reads += rd_;
		my_hits += hh.hit;
	}
	if (counters)
		warp_add_counters(counters, my_steps, my_reads, my_hits);
}

__global__ void k_trace(DevPool P, u32 root, const float *o, const float *d, u32 n, hd_hit *out) {
	for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
		out[i] = trace_one(P, root, o[3 * i], o[3 * i + 1], o[3 * i + 2], d[3 * i], d[3 * i + 1], d[3 * i + 2]);
}

// Camera_GenRay (shader/src/trace.frag:366-370) at pixel centres, then the traversal.
// counters (optional): [0] += loop iterations, [1] += node words read, [2] += hits.
__global__ void k_trace_pinhole(DevPool P, u32 root, const hd_camera *cams, u32 n_cams, u32 w, u32 h, hd_hit *out,
                                unsigned long long *counters) {
	const u64 per = (u64)w * h, total = per * n_cams;
	u64 my_steps = 0, my_reads = 0, my_hits = 0;
	for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x) {
		const u32 c = (u32)(i / per);
		const u32 px = (u32)(i % per % w), py = (u32)(i % per / w);
		const hd_camera cam = cams[c];
		float d[3];
		pinhole_dir(cam, px, py, w, h, d);
		u32 st_, rd_;
		const hd_hit hh = trace_one(P, root, cam.position[0], cam.position[1], cam.position[2], d[0], d[1], d[2], &st_, &rd_);
		out[i] = hh;
		my_steps += st_;
		my_reads += rd_;
		my_hits += hh.hit;
	}
	if (counters) // one atomic per warp and counter
		warp_add_counters(counters, my_steps, my_reads, my_hits);
}

// The pinhole traversal, stackless (ParentRing), with every warp on an 8 x 4
// tile of pixels instead of 32 pixels of one row: neighbouring rays walk the
// same nodes, so a warp's loads coalesce and its lanes stay in step longer.
// Same hit records as k_trace_pinhole, at the same output positions.
constexpr u32 kTileW = 8, kTileH = 4;
__global__ void k_trace_pinhole_stackless(DevPool P, u32 root, const hd_camera *cams, u32 n_cams, u32 w, u32 h,
                                          hd_hit *out, unsigned long long *counters) {
	const u32 tx = (w + kTileW - 1) / kTileW, ty = (h + kTileH - 1) / kTileH;
	const u64 tiles = (u64)tx * ty, total = tiles * 32u * n_cams;
	u64 my_steps = 0, my_reads = 0, my_hits = 0;
	for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x) {
		const u32 c = (u32)(i / (tiles * 32u));
		const u64 t = i % (tiles * 32u) / 32u;
		const u32 lane = (u32)(i & 31u);
		const u32 px = (u32)(t % tx) * kTileW + (lane % kTileW), py = (u32)(t / tx) * kTileH + (lane / kTileW);
		if (px >= w || py >= h)
			continue;
		const hd_camera cam = cams[c];
		float d[3];
		pinhole_dir(cam, px, py, w, h, d);
		u32 st_ = 0, rd_ = 0;
		const hd_hit hh = trace_core<false, true>(P, root, cam.position[0], cam.position[1], cam.position[2], d[0], d[1],
		                                          d[2], 0.0f, 0.0f, &st_, &rd_, nullptr);
		out[(u64)c * w * h + (u64)py * w + px] = hh;
		my_steps += st_;
		my_reads += rd_;
		my_hits += hh.hit;
	}
	if (counters)
		warp_add_counters(counters, my_steps, my_reads, my_hits);
}

} // namespace

extern "C" {

hd_status hd_trace(hd_pool *pool, uint32_t root, const float *origins, const float *dirs, uint32_t n, hd_hit *out,
                   void *stream) {
	if (!pool || (n && (!origins || !dirs || !out)))
		return HD_ERR_INVALID_ARG;
	if (!n)
		return HD_OK;
	std::lock_guard<std::mutex> lk(pool->mtx);
	if (cudaSetDevice(pool->device) != cudaSuccess)
		return HD_ERR_CUDA;
	cudaStream_t st = (cudaStream_t)stream;
	float *d_o = nullptr, *d_d = nullptr;
	hd_hit *d_out = nullptr;
	hd_status s = HD_OK;
	if (cudaMalloc(&d_o, n * 12ull) != cudaSuccess || cudaMalloc(&d_d, n * 12ull) != cudaSuccess ||
	    cudaMalloc(&d_out, n * sizeof(hd_hit)) != cudaSuccess)
		s = HD_ERR_CUDA;
	if (!s && (cudaStreamWaitEvent(st, pool->ws_free, 0) != cudaSuccess ||
	           cudaMemcpyAsync(d_o, origins, n * 12ull, cudaMemcpyHostToDevice, st) != cudaSuccess ||
	           cudaMemcpyAsync(d_d, dirs, n * 12ull, cudaMemcpyHostToDevice, st) != cudaSuccess))
		s = HD_ERR_CUDA;
	if (!s) {
		const uint32_t grid = std::max(1u, std::min((n + 255u) / 256u, (uint32_t)pool->num_sms * 16u));
		k_trace<<<grid, 256, 0, st>>>(pool->P, root, d_o, d_d, n, d_out);
		if (cudaGetLastError() != cudaSuccess ||
		    cudaMemcpyAsync(out, d_out, n * sizeof(hd_hit), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
		    cudaStreamSynchronize(st) != cudaSuccess)
			s = HD_ERR_CUDA;
	}
	cudaFree(d_o);
	cudaFree(d_d);
	cudaFree(d_out);
	return s;
}

hd_status hd_trace_pinhole_async(hd_pool *pool, uint32_t root, const hd_camera *cameras, uint32_t n_cameras,
                                 uint32_t width, uint32_t height, hd_hit *d_out, uint64_t *d_counters, void *stream) {
	if (!pool || !cameras || !d_out || !n_cameras || !width || !height)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	if (cudaSetDevice(pool->device) != cudaSuccess)
		return HD_ERR_CUDA;
	cudaStream_t st = (cudaStream_t)stream;
	if (cudaStreamWaitEvent(st, pool->ws_free, 0) != cudaSuccess)
		return HD_ERR_CUDA;
	hd_camera *d_cams = nullptr;
	if (cudaMallocAsync((void **)&d_cams, n_cameras * sizeof(hd_camera), st) != cudaSuccess)
		return HD_ERR_CUDA;
	hd_status s = HD_OK;
	if (cudaMemcpyAsync(d_cams, cameras, n_cameras * sizeof(hd_camera), cudaMemcpyHostToDevice, st) != cudaSuccess)
		s = HD_ERR_CUDA;
	if (!s)
		s = hd_launch_pinhole(pool, root, d_cams, n_cameras, width, height, d_out, d_counters, st);
	cudaFreeAsync(d_cams, st);
	return s;
}

hd_status hd_trace_pinhole_stackless_async(hd_pool *pool, uint32_t root, const hd_camera *cameras,
                                           uint32_t n_cameras, uint32_t width, uint32_t height, hd_hit *d_out,
                                           uint64_t *d_counters, void *stream) {
	if (!pool || !cameras || !d_out || !n_cameras || !width || !height)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	if (cudaSetDevice(pool->device) != cudaSuccess)
		return HD_ERR_CUDA;
	cudaStream_t st = (cudaStream_t)stream;
	if (cudaStreamWaitEvent(st, pool->ws_free, 0) != cudaSuccess)
		return HD_ERR_CUDA;
	hd_camera *d_cams = nullptr;
	if (cudaMallocAsync((void **)&d_cams, n_cameras * sizeof(hd_camera), st) != cudaSuccess)
		return HD_ERR_CUDA;
	hd_status s = HD_OK;
	if (cudaMemcpyAsync(d_cams, cameras, n_cameras * sizeof(hd_camera), cudaMemcpyHostToDevice, st) != cudaSuccess)
		s = HD_ERR_CUDA;
	if (!s)
		s = hd_launch_pinhole_stackless(pool, root, d_cams, n_cameras, width, height, d_out, d_counters, st);
	cudaFreeAsync(d_cams, st);
	return s;
}

float hd_projection_factor(float fov_y, uint32_t height, uint32_t divisor) {
	// src/rg/TracePass.cpp:114-118 (divisor 1), src/rg/BeamPass.cpp:90-94 (divisor 8)
	const float inv_2tan_half_fov = 1.0f / (2.0f * std::tan(0.5f * fov_y));
	const float screen_tolerance = 1.0f / (float(height) / float(divisor));
	return inv_2tan_half_fov / screen_tolerance;
}

hd_status hd_trace_pinhole_lod_async(hd_pool *pool, uint32_t root, const hd_camera *cameras, uint32_t n_cameras,
                                     uint32_t width, uint32_t height, float proj_factor, float beam_proj_factor,
                                     hd_hit *d_out, uint64_t *d_counters, void *stream) {
	if (!pool || !cameras || !d_out || !n_cameras || !width || !height || !(proj_factor > 0.0f))
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(pool->mtx);
	if (cudaSetDevice(pool->device) != cudaSuccess)
		return HD_ERR_CUDA;
	cudaStream_t st = (cudaStream_t)stream;
	if (cudaStreamWaitEvent(st, pool->ws_free, 0) != cudaSuccess)
		return HD_ERR_CUDA;
	const bool use_beam = beam_proj_factor > 0.0f;
	const uint32_t bw = (width + kBeamBlock - 1) / kBeamBlock, bh = (height + kBeamBlock - 1) / kBeamBlock;
	hd_camera *d_cams = nullptr;
	float *d_beam = nullptr;
	if (cudaMallocAsync((void **)&d_cams, n_cameras * sizeof(hd_camera), st) != cudaSuccess)
		return HD_ERR_CUDA;
	hd_status s = HD_OK;
	if (use_beam && cudaMallocAsync((void **)&d_beam, (uint64_t)n_cameras * bw * bh * 4, st) != cudaSuccess)
		s = HD_ERR_CUDA;
	if (!s && cudaMemcpyAsync(d_cams, cameras, n_cameras * sizeof(hd_camera), cudaMemcpyHostToDevice, st) != cudaSuccess)
		s = HD_ERR_CUDA;
	unsigned long long *ctr = reinterpret_cast<unsigned long long *>(d_counters);
	if (!s && use_beam) {
		const uint64_t nb = (uint64_t)n_cameras * bw * bh;
		const uint32_t grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((nb + 255) / 256, pool->num_sms * 16ull));
		k_beam<<<grid, 256, 0, st>>>(pool->P, root, d_cams, n_cameras, bw, bh, beam_proj_factor, d_beam, ctr);
		pool->kernel_launches++;
	}
	if (!s) {
		const uint64_t total = (uint64_t)width * height * n_cameras;
		const uint32_t grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((total + 255) / 256, pool->num_sms * 16ull));
		k_trace_pinhole_lod<<<grid, 256, 0, st>>>(pool->P, root, d_cams, n_cameras, width, height, proj_factor, d_beam,
		                                          bw, bh, d_out, ctr);
		pool->kernel_launches++;
		if (cudaGetLastError() != cudaSuccess)
			s = HD_ERR_CUDA;
	}
	if (d_beam)
		cudaFreeAsync(d_beam, st);
	cudaFreeAsync(d_cams, st);
	return s;
}

} // extern "C"

// Launchers shared with the serving loop: stream-ordered, no wait for edit
// passes of other streams (the caller traces a root whose pass has completed).
hd_status hd_launch_pinhole(hd_pool *pool, uint32_t root, const hd_camera *d_cams, uint32_t n_cameras, uint32_t width,
                            uint32_t height, hd_hit *d_out, uint64_t *d_counters, cudaStream_t st) {
	const uint64_t total = (uint64_t)width * height * n_cameras;
	const uint32_t grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((total + 255) / 256, pool->num_sms * 16ull));
	k_trace_pinhole<<<grid, 256, 0, st>>>(pool->P, root, d_cams, n_cameras, width, height, d_out,
	                                      reinterpret_cast<unsigned long long *>(d_counters));
	pool->kernel_launches++;
	return cudaGetLastError() == cudaSuccess ? HD_OK : HD_ERR_CUDA;
}

hd_status hd_launch_pinhole_stackless(hd_pool *pool, uint32_t root, const hd_camera *d_cams, uint32_t n_cameras,
                                      uint32_t width, uint32_t height, hd_hit *d_out, uint64_t *d_counters,
                                      cudaStream_t st) {
	const uint64_t lanes = (uint64_t)((width + kTileW - 1) / kTileW) * ((height + kTileH - 1) / kTileH) * 32u * n_cameras;
	const uint32_t grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((lanes + 255) / 256, pool->num_sms * 16ull));
	k_trace_pinhole_stackless<<<grid, 256, 0, st>>>(pool->P, root, d_cams, n_cameras, width, height, d_out,
	                                                reinterpret_cast<unsigned long long *>(d_counters));
	pool->kernel_launches++;
	return cudaGetLastError() == cudaSuccess ? HD_OK : HD_ERR_CUDA;
}

hd_status hd_launch_rays(hd_pool *pool, uint32_t root, const float *d_o, const float *d_d, uint32_t n, hd_hit *d_out,
                         cudaStream_t st) {
	const uint32_t grid = std::max(1u, std::min((n + 255u) / 256u, (uint32_t)pool->num_sms * 16u));
	k_trace<<<grid, 256, 0, st>>>(pool->P, root, d_o, d_d, n, d_out);
	pool->kernel_launches++;
	return cudaGetLastError() == cudaSuccess ? HD_OK : HD_ERR_CUDA;
}
