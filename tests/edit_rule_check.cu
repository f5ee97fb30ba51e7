// edit_rule_check.cu -- host-side check of the per-node rules of the edit kernels.
//
// The edit kernels decide every node from the classification of the SphereEditor
// and AABBEditor EditNode (src/main.cpp:36-47,77-106) and every partly covered
// leaf from VoxelInRange (src/main.cpp:55-57,121-126) in the voxel order of
// NodeCoord.hpp:32-43.  The functions that do it are __host__ __device__, so this
// program runs the kernels' own code on the CPU and compares it with rules
// written here from the reference's predicates:
//   * the leaf rule (classify at leaf granularity, then shape_mask for a partial
//     leaf) against a per-voxel brute force: the box mask's per-axis runs and
//     spread multiplies for all 16^3 combinations of axis masks and for every run
//     of a small coordinate range; boxes (empty, thin, large) and spheres sampled
//     around their surfaces, in the 32-bit paths (centre and bounds below 2^15;
//     the sign-bit mask for r2 <= 2^29, the compare mask up to 2^30) and the
//     64-bit ones (coordinates up to 2^21, r2 above 2^30);
//   * the expand kernel's classify_children (the 8 children of a node against
//     one edit, each axis's terms shared by the children on the same half)
//     against classify of each child, at every cell size from 4 to 2^20 voxels.
// Exit status 0 and "ok <counts>" on success; the first mismatches are printed.
//
// `edit_rule_check hashes IN OUT` hashes nodes the way the dedup kernel does
// (Murmur over an inner node's words finished with its length; hash_leaf of a
// leaf's 64 bits, low word first) for records of IN (kind 0 inner / 1 leaf,
// length, words; uint32) and writes one uint32 per record to OUT, for a test
// to compare with the oracle's hashes (Hasher.hpp:21-48).
#include "../vkhashdag_gb300/csrc/hd_device.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>

using namespace hd;

static u64 g_state = 0x853c49e6748fea9bull;
static u64 next_u64() { // splitmix64
	u64 z = (g_state += 0x9e3779b97f4a7c15ull);
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
	return z ^ (z >> 31);
}
static u32 below(u32 n) { return n ? (u32)(next_u64() % n) : 0u; }
static double unit() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

static u32 vx(u32 i) { return ((i >> 2) & 2u) | (i & 1u); }
static u32 vy(u32 i) { return ((i >> 3) & 2u) | ((i >> 1) & 1u); }
static u32 vz(u32 i) { return ((i >> 4) & 2u) | ((i >> 2) & 1u); }

// The reference's per-voxel predicates, in exact integer arithmetic.
static bool inside(const hd_edit_desc &e, u32 x, u32 y, u32 z) {
	if (e.shape == HD_SHAPE_AABB)
		return x >= e.p0[0] && x < e.p1[0] && y >= e.p0[1] && y < e.p1[1] && z >= e.p0[2] && z < e.p1[2];
	const long long dx = (long long)x - e.p0[0], dy = (long long)y - e.p0[1], dz = (long long)z - e.p0[2];
	return (unsigned long long)(dx * dx + dy * dy + dz * dz) <= e.r2;
}

static u64 brute(const hd_edit_desc &e, u32 ox, u32 oy, u32 oz) {
	u64 m = 0;
	for (u32 i = 0; i < 64; ++i)
		if (inside(e, ox + vx(i), oy + vy(i), oz + vz(i)))
			m |= 1ull << i;
	return m;
}

static int g_fail = 0;
static unsigned long long g_checked[3] = {0, 0, 0}; // leaves classified none / partial / full

static void check_leaf(const hd_edit_desc &e, u32 lx, u32 ly, u32 lz) {
	const u32 cls = classify(e, 2u, lx, ly, lz);
	const u64 got = cls == kClsNone ? 0ull : cls == kClsFull ? ~0ull : shape_mask(e, lx << 2, ly << 2, lz << 2);
	const u64 want = brute(e, lx << 2, ly << 2, lz << 2);
	++g_checked[cls];
	bool voxel_ok = true;
	for (u32 i = 0; i < 64; ++i)
		voxel_ok &= voxel_in(e, (lx << 2) + vx(i), (ly << 2) + vy(i), (lz << 2) + vz(i)) == (((want >> i) & 1u) != 0);
	if ((got != want || !voxel_ok) && g_fail++ < 10)
		std::printf("mismatch shape %u p0 (%u,%u,%u) p1 (%u,%u,%u) r2 %llu leaf (%u,%u,%u) cls %u got %016llx want %016llx%s\n",
		            e.shape, e.p0[0], e.p0[1], e.p0[2], e.p1[0], e.p1[1], e.p1[2], (unsigned long long)e.r2, lx, ly, lz,
		            cls, (unsigned long long)got, (unsigned long long)want, voxel_ok ? "" : " (voxel_in differs)");
}

static void check_spread() {
	for (u32 mx = 0; mx < 16; ++mx)
		for (u32 my = 0; my < 16; ++my)
			for (u32 mz = 0; mz < 16; ++mz) {
				u64 want = 0;
				for (u32 i = 0; i < 64; ++i)
					if (((mx >> vx(i)) & 1u) && ((my >> vy(i)) & 1u) && ((mz >> vz(i)) & 1u))
						want |= 1ull << i;
				const u64 got = spread_x(mx) & spread_y(my) & spread_z(mz);
				if (got != want && g_fail++ < 10)
					std::printf("spread mismatch %x %x %x: %016llx vs %016llx\n", mx, my, mz, (unsigned long long)got,
					            (unsigned long long)want);
			}
	const u32 big[] = {0x7FFFFFF0u, 0x7FFFFFFCu, 0xFFFFFFF0u, 0xFFFFFFFBu};
	for (u32 o = 0; o < 40; ++o)
		for (u32 lo = 0; lo < 48; ++lo)
			for (u32 hi = 0; hi < 48; ++hi) {
				u32 want = 0;
				for (u32 k = 0; k < 4; ++k)
					want |= (u32)(lo <= o + k && o + k < hi) << k;
				const u32 got = axis_run(o, lo, hi);
				if (got != want && g_fail++ < 10)
					std::printf("axis_run mismatch o %u lo %u hi %u: %x vs %x\n", o, lo, hi, got, want);
			}
	for (u32 o : big)
		for (u32 dl = 0; dl < 12; ++dl)
			for (u32 dh = 0; dh < 12; ++dh) {
				const u32 lo = o - 4 + dl, hi = o - 4 + dh;
				u32 want = 0;
				for (u32 k = 0; k < 4; ++k)
					want |= (u32)(lo <= o + k && o + k < hi) << k;
				if (axis_run(o, lo, hi) != want && g_fail++ < 10)
					std::printf("axis_run mismatch o %u lo %u hi %u\n", o, lo, hi);
			}
}

// Boxes of sides 0..max_side (empty, thin and large), leaves sampled over the
// box's bounds widened by two leaves.
static void check_boxes(u32 world, u32 max_side, int n_edits, int leaves_per_edit) {
	for (int t = 0; t < n_edits; ++t) {
		hd_edit_desc e{};
		e.shape = HD_SHAPE_AABB;
		for (int a = 0; a < 3; ++a) {
			const u32 side = (t % 7 == 0) ? below(3) : (u32)std::exp(unit() * std::log((double)max_side + 1.0));
			e.p0[a] = below(world - side);
			e.p1[a] = (t % 11 == 0) ? e.p0[a] - below(3) : e.p0[a] + side; // some empty or inverted
		}
		for (int s = 0; s < leaves_per_edit; ++s) {
			u32 l[3];
			for (int a = 0; a < 3; ++a) {
				const u32 lo = e.p0[a] / 4 > 2 ? e.p0[a] / 4 - 2 : 0, hi = e.p1[a] / 4 + 2;
				l[a] = lo + below(hi > lo ? hi - lo + 1 : 1);
				if ((s & 3) == 0) // a leaf on a face of the box
					l[a] = (s & 4 ? e.p0[a] : e.p1[a]) / 4;
			}
			check_leaf(e, l[0], l[1], l[2]);
		}
	}
}

// Spheres with centres below `world` and radii log-uniform up to max_r; the
// leaves sampled at random directions within a few voxels of the surface, and
// some uniformly over the bounding box.
static void check_spheres(u32 world, double max_r, int n_edits, int leaves_per_edit, bool r2_exact_edges) {
	for (int t = 0; t < n_edits; ++t) {
		hd_edit_desc e{};
		e.shape = HD_SHAPE_SPHERE;
		for (int a = 0; a < 3; ++a)
			e.p0[a] = below(world);
		const double r = std::exp(unit() * std::log(max_r));
		e.r2 = (u64)(r * r) + below(3);
		if (r2_exact_edges && t % 4 == 0) // 2^30 - 1, 2^30, 2^30 + 1, 2^29 - 1, 2^29, 2^29 + 1
			e.r2 = (1ull << (t / 4 % 2 ? 29 : 30)) + (u64)(t / 8 % 3) - 1;
		const double rr = std::sqrt((double)e.r2);
		for (int s = 0; s < leaves_per_edit; ++s) {
			double d[3], n = 0;
			for (int a = 0; a < 3; ++a) {
				d[a] = unit() * 2.0 - 1.0;
				n += d[a] * d[a];
			}
			n = std::sqrt(n) + 1e-12;
			const double dist = (s & 3) ? rr + (unit() * 12.0 - 6.0) : rr * unit() * 1.2;
			long long q[3];
			bool ok = true;
			for (int a = 0; a < 3; ++a) {
				q[a] = (long long)std::floor(e.p0[a] + d[a] / n * dist);
				ok &= q[a] >= 0 && q[a] < (1ll << 31) - 8;
			}
			if (ok)
				check_leaf(e, (u32)(q[0] >> 2), (u32)(q[1] >> 2), (u32)(q[2] >> 2));
		}
	}
}

// Nodes of cell size 2^(shift+1) near the edit (and some anywhere in the world):
// classify_children packs, per child c, classify(e, shift, 2p + half(c)).
static unsigned long long g_children[3] = {0, 0, 0}; // children classified none / partial / full
static void check_children(const hd_edit_desc &e, u32 world_bits, int n_nodes) {
	for (int s = 0; s < n_nodes; ++s) {
		const u32 shift = 1u + below(world_bits - 1u); // child cell 2^shift, node 2^(shift+1) <= world
		const u32 nbits = world_bits - shift - 1u;      // node coordinates below 2^nbits
		u32 p[3];
		for (int a = 0; a < 3; ++a) {
			u32 v;
			if (s & 1) {
				v = below(1u << world_bits);
			} else { // near the edit's bounds
				const u32 c = e.shape == HD_SHAPE_AABB ? ((s & 2) ? e.p0[a] : e.p1[a]) : e.p0[a];
				const u32 r = e.shape == HD_SHAPE_AABB ? 0u : (u32)std::sqrt((double)e.r2);
				const long long off = (long long)below(2u * r + 16u) - (long long)r - 8;
				long long q = (long long)c + off;
				q = q < 0 ? 0 : (q >= (1ll << world_bits) ? (1ll << world_bits) - 1 : q);
				v = (u32)q;
			}
			p[a] = (v >> (shift + 1u)) & ((1u << nbits) - 1u);
		}
		const u32 got = classify_children(e, shift, p[0], p[1], p[2]);
		u32 want = 0;
		for (u32 c = 0; c < 8; ++c)
			want |= classify(e, shift, 2u * p[0] + (c & 1u), 2u * p[1] + ((c >> 1) & 1u), 2u * p[2] + ((c >> 2) & 1u))
			        << (2u * c);
		for (u32 c = 0; c < 8; ++c)
			++g_children[(want >> (2u * c)) & 3u];
		if (got != want && g_fail++ < 10)
			std::printf("children mismatch shape %u p0 (%u,%u,%u) p1 (%u,%u,%u) r2 %llu shift %u node (%u,%u,%u): %04x vs %04x\n",
			            e.shape, e.p0[0], e.p0[1], e.p0[2], e.p1[0], e.p1[1], e.p1[2], (unsigned long long)e.r2, shift,
			            p[0], p[1], p[2], got, want);
	}
}

static void check_children_all(u32 world_bits, double max_r, int n_edits) {
	const u32 world = 1u << world_bits;
	for (int t = 0; t < n_edits; ++t) {
		hd_edit_desc e{};
		if (t & 1) {
			e.shape = HD_SHAPE_AABB;
			for (int a = 0; a < 3; ++a) {
				const u32 side = (u32)std::exp(unit() * std::log(max_r * 2.0 + 1.0));
				e.p0[a] = below(world - (side < world ? side : world - 1u));
				e.p1[a] = (t % 13 == 1) ? e.p0[a] : e.p0[a] + side;
			}
		} else {
			e.shape = HD_SHAPE_SPHERE;
			for (int a = 0; a < 3; ++a)
				e.p0[a] = below(world);
			const double r = std::exp(unit() * std::log(max_r));
			e.r2 = (u64)(r * r) + below(3);
			if (t % 8 == 0)
				e.r2 = (1ull << 30) + (u64)(t / 8 % 3) - 1;
			if (t % 16 == 2)
				e.r2 = 0xFFFFFFFFull + (u64)(t / 16 % 3) - 1; // the 32-bit clamp's edge
		}
		check_children(e, world_bits, 64);
	}
}

static int hashes(const char *in, const char *out) {
	FILE *f = std::fopen(in, "rb"), *g = std::fopen(out, "wb");
	if (!f || !g)
		return 2;
	u32 kind, len, w[9];
	while (std::fread(&kind, 4, 1, f) == 1 && std::fread(&len, 4, 1, f) == 1) {
		if (len < 1 || len > 9 || std::fread(w, 4, len, f) != len)
			return 2;
		u32 h;
		if (kind == 1) {
			h = hash_leaf((u64)w[0] | ((u64)w[1] << 32));
		} else {
			Murmur m;
			for (u32 k = 0; k < len; ++k)
				m.add(w[k]);
			h = m.finish(len);
		}
		std::fwrite(&h, 4, 1, g);
	}
	std::fclose(f);
	std::fclose(g);
	std::printf("ok hashes\n");
	return 0;
}

int main(int argc, char **argv) {
	if (argc == 4 && std::strcmp(argv[1], "hashes") == 0)
		return hashes(argv[2], argv[3]);
	check_spread();
	check_boxes(1u << 15, 2048, 4000, 64);
	check_boxes(1u << 21, 1u << 20, 2000, 64);
	check_spheres(1u << 15, 16384.0, 4000, 64, false); // 32-bit classify and mask
	check_spheres(1u << 15, 32768.0, 1000, 64, true);  // r2 around 2^29 and 2^30
	check_spheres(1u << 15, 24000.0, 2000, 64, false); // r2 up to 2^29 and a little above
	check_spheres(1u << 21, 32768.0, 2000, 64, true);  // 64-bit classify, 32-bit mask
	check_spheres(1u << 21, 1u << 20, 2000, 64, false); // 64-bit classify and mask
	check_children_all(15, 16384.0, 4000);   // 32-bit child classification
	check_children_all(21, 1u << 20, 4000);  // 64-bit
	if (g_fail) {
		std::printf("FAILED %d\n", g_fail);
		return 1;
	}
	std::printf("ok none %llu partial %llu full %llu child_none %llu child_partial %llu child_full %llu\n",
	            g_checked[0], g_checked[1], g_checked[2], g_children[0], g_children[1], g_children[2]);
	return 0;
}
