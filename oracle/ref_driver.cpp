// ref_driver.cpp -- runs the reference's own hashdag header library.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh against the
// reference headers (include/hashdag/*.hpp, dep/libfork, dep/glm) where the
// reference tree is present, into oracle/_ref/.  It executes the reference's
// NodePoolBase::Edit, NodePoolThreadedEdit::ThreadedEdit,
// NodePoolBase::upsert_inner_node / upsert_leaf, NodePoolThreadedGC::ThreadedGC
// and NodePoolTraversal::Traversal on the product's host pool mirror (whose
// storage hooks follow src/DAGNodePool.hpp:56-69), and dumps the resulting pool, so the
// oracle restatement can be pinned against the reference and golden fixtures
// can be generated.  The editors restate the stateless SphereEditor<kFill/kDig>
// and AABBEditor of src/main.cpp:32-150 (they live in the application, not the
// library) plus an AABB dig by symmetry.
//
// Protocol (all little-endian uint32 unless noted), input file:
//   magic 'HDRQ', mode (0 edit, 1 threaded edit, 2 upsert, 3 trace-after-edit,
//   4 edit then garbage-collect),
//   wbpp, pbpb, node_levels, hasher, bucket_bits[node_levels],
//   threads, max_task_level, n_edits, edits[n_edits] (40 bytes each),
//   mode 2: n_ops, then per op: level, len, words[len]
//   mode 3: n_rays, then origins[3n] and dirs[3n] (float)
//   mode 4: n_keep, keep[n_keep] (keep the root after edit keep[i]; the roots
//           are the GC roots, collected by ThreadedGC on a pool of `threads`
//           workers, one for the deterministic layout of the golden cases)
//   mode 5 (colour edits through VBREditorWrapper): color_leaf_level,
//           keep_history, per edit: kind (0 stateless, 1 VBR fill, 2 VBR
//           paint), colors, weight, bits_per_weight; then n_queries and
//           queries[3n] (voxel coordinates) for colour lookups
// output file:
//   magic 'HDRS', root, ok, elapsed_ns (uint64), filled[node_levels],
//   total_buckets, bucket_words[total_buckets], n_pages, then per page: id, words[wpp]
//   mode 2: n_ops, ptrs[n_ops] (after the pool dump)
//   mode 3: n_rays, per ray: hit, pos[3] (float); then the traversals' time
//           (uint64 ns, one thread)
//   mode 4: the dump is the pool after GC; then n_keep, roots before[n_keep],
//           roots after[n_keep], the collection's time (uint64 ns)
//   mode 5: colour root, n_nodes, nodes[8 n_nodes], n_leaf_words,
//           leaf_words[n], then per query: has_value, colors, weight,
//           bits_per_weight, rgb[3] (float, VBRColor::Get()); then the time
//           of each edit (uint64 ns)

#include <hashdag/NodePool.hpp>
#include <hashdag/NodePoolThreadedEdit.hpp>
#include <hashdag/NodePoolThreadedGC.hpp>
#include <hashdag/NodePoolTraversal.hpp>
#include <hashdag/VBREditor.hpp>
#include <parallel_hashmap/phmap.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "../include/hashdag_gpu.h"
#include "../include/hashdag_host_mirror.hpp"

struct ZeroHasher {
	inline uint32_t operator()(auto &&) const { return 0; }
};

// the map/set types the application instantiates the GC with (src/DAGNodePool.hpp:26-29)
template <typename K, typename V> using GcMap = phmap::flat_hash_map<K, V>;
template <typename K> using GcSet = phmap::flat_hash_set<K>;

// The pool's storage is the product's host mirror (include/hashdag_host_mirror.hpp,
// whose hooks follow src/DAGNodePool.hpp:56-74): every run of the reference's
// algorithms below goes through those hooks, and the static_asserts check that
// the mirror satisfies the reference's storage concepts.
template <typename HasherT>
struct RefPool final : public hashdag_gb300::HostPoolMirror,
                       public hashdag::NodePoolBase<RefPool<HasherT>, uint32_t>,
                       public hashdag::NodePoolThreadedEdit<RefPool<HasherT>, uint32_t>,
                       public hashdag::NodePoolThreadedGC<RefPool<HasherT>, uint32_t, GcMap, GcSet>,
                       public hashdag::NodePoolTraversal<RefPool<HasherT>, uint32_t> {
	using WordSpanHasher = HasherT;
	using Base = hashdag::NodePoolBase<RefPool<HasherT>, uint32_t>;

	RefPool(const hashdag::Config<uint32_t> &config, const hd_config &hc)
	    : hashdag_gb300::HostPoolMirror(hc), Base(config) {}
	~RefPool() final = default;
};
static_assert(hashdag::NodePool<RefPool<hashdag::MurmurHasher32>, uint32_t>);
static_assert(hashdag::ThreadedNodePool<RefPool<hashdag::MurmurHasher32>, uint32_t>);
static_assert(hashdag::GCNodePool<RefPool<hashdag::MurmurHasher32>, uint32_t>);

// Stateless editors (src/main.cpp:32-150) for one hd_edit_desc.
struct DescEditor {
	hd_edit_desc e;
	inline hashdag::EditType EditNode(const hashdag::Config<uint32_t> &config, const hashdag::NodeCoord<uint32_t> &coord,
	                                  hashdag::NodePointer<uint32_t>) const {
		auto lb = coord.GetLowerBoundAtLevel(config.GetVoxelLevel()), ub = coord.GetUpperBoundAtLevel(config.GetVoxelLevel());
		if (e.shape == HD_SHAPE_AABB) {
			glm::u32vec3 mn{e.p0[0], e.p0[1], e.p0[2]}, mx{e.p1[0], e.p1[1], e.p1[2]};
			if (glm::any(glm::lessThanEqual(ub, mn)) || glm::any(glm::greaterThanEqual(lb, mx)))
				return hashdag::EditType::kNotAffected;
			if (glm::all(glm::greaterThanEqual(lb, mn)) && glm::all(glm::lessThanEqual(ub, mx)))
				return e.op == HD_OP_DIG ? hashdag::EditType::kClear : hashdag::EditType::kFill;
			return hashdag::EditType::kProceed;
		}
		glm::u32vec3 center{e.p0[0], e.p0[1], e.p0[2]};
		glm::i64vec3 lb_dist = glm::i64vec3{lb} - glm::i64vec3(center);
		glm::i64vec3 ub_dist = glm::i64vec3{ub} - glm::i64vec3(center);
		glm::u64vec3 lb_dist_2 = lb_dist * lb_dist;
		glm::u64vec3 ub_dist_2 = ub_dist * ub_dist;
		glm::u64vec3 max_dist_2 = glm::max(lb_dist_2, ub_dist_2);
		uint64_t max_n2 = max_dist_2.x + max_dist_2.y + max_dist_2.z;
		if (max_n2 <= e.r2)
			return e.op == HD_OP_DIG ? hashdag::EditType::kClear : hashdag::EditType::kFill;
		uint64_t min_n2 = 0;
		if (lb_dist.x > 0)
			min_n2 += lb_dist_2.x;
		if (ub_dist.x < 0)
			min_n2 += ub_dist_2.x;
		if (lb_dist.y > 0)
			min_n2 += lb_dist_2.y;
		if (ub_dist.y < 0)
			min_n2 += ub_dist_2.y;
		if (lb_dist.z > 0)
			min_n2 += lb_dist_2.z;
		if (ub_dist.z < 0)
			min_n2 += ub_dist_2.z;
		return min_n2 > e.r2 ? hashdag::EditType::kNotAffected : hashdag::EditType::kProceed;
	}
	inline bool EditVoxel(const hashdag::Config<uint32_t> &, const hashdag::NodeCoord<uint32_t> &coord, bool voxel) const {
		bool in;
		if (e.shape == HD_SHAPE_AABB) {
			glm::u32vec3 mn{e.p0[0], e.p0[1], e.p0[2]}, mx{e.p1[0], e.p1[1], e.p1[2]};
			in = glm::all(glm::greaterThanEqual(coord.pos, mn)) && glm::all(glm::lessThan(coord.pos, mx));
		} else {
			glm::i64vec3 d = glm::i64vec3{coord.pos.x, coord.pos.y, coord.pos.z} -
			                 glm::i64vec3(glm::u32vec3{e.p0[0], e.p0[1], e.p0[2]});
			uint64_t n2 = d.x * d.x + d.y * d.y + d.z * d.z;
			in = n2 <= e.r2;
		}
		return e.op == HD_OP_DIG ? (voxel && !in) : (voxel || in);
	}
};

// Colour octree with the behaviour of the application's DAGColorPool
// (src/DAGColorPool.hpp:20-218) on plain vectors instead of Vulkan paged
// buffers: tagged 32-bit pointers (2-bit tag: node, colour, leaf, null; 30-bit
// data), nodes of 8 child pointers appended in JoinNode order, VBR leaf chunks
// in one word vector ([block size][macro count][block count][weight words]
// [macro blocks][block headers][weight words]), rewritten in place when
// keep_history is off and the new chunk fits, else appended with doubled room.
struct RefColorPool {
	struct Pointer {
		static constexpr uint32_t kDataBits = 30u;
		enum class Tag { kNode = 0, kColor, kLeaf, kNull };
		uint32_t pointer;
		Pointer() : Pointer(Tag::kNull, 0u) {}
		Pointer(Tag tag, uint32_t data) : pointer{(static_cast<uint32_t>(tag) << kDataBits) | data} {}
		Tag GetTag() const { return static_cast<Tag>(pointer >> kDataBits); }
		uint32_t GetData() const { return pointer & ((1u << kDataBits) - 1u); }
		bool operator==(const Pointer &r) const { return pointer == r.pointer; }
	};
	using Node = std::array<Pointer, 8>;
	using Chunk = hashdag::VBRChunk<uint32_t, hashdag::VBRWriterContainer>;
	std::vector<Node> nodes;
	std::vector<uint32_t> leaves;
	uint32_t leaf_level = 0;
	bool keep_history = false;

	Pointer GetChild(Pointer ptr, auto idx) const {
		return ptr.GetTag() == Pointer::Tag::kNode ? nodes[ptr.GetData()][idx]
		                                           : (ptr.GetTag() == Pointer::Tag::kColor ? ptr : Pointer{});
	}
	static hashdag::VBRColor GetFill(Pointer ptr) {
		return ptr.GetTag() == Pointer::Tag::kColor ? hashdag::VBRColor{hashdag::RGB8Color{ptr.GetData()}}
		                                            : hashdag::VBRColor{};
	}
	Pointer SetNode(Pointer ptr, std::span<const Pointer, 8> ch) {
		if (std::ranges::all_of(ch, [](Pointer p) { return p.GetTag() == Pointer::Tag::kNull; }))
			return {};
		if (Pointer c = ch[0];
		    c.GetTag() == Pointer::Tag::kColor && std::ranges::all_of(ch.subspan(1), [c](Pointer p) { return p == c; }))
			return c;
		if (ptr.GetTag() == Pointer::Tag::kNode && std::ranges::equal(nodes[ptr.GetData()], ch))
			return ptr;
		Node n;
		std::ranges::copy(ch, n.begin());
		nodes.push_back(n);
		return Pointer{Pointer::Tag::kNode, (uint32_t)(nodes.size() - 1)};
	}
	static Pointer ClearNode(Pointer) { return Pointer{}; }
	static Pointer FillNode(Pointer, hashdag::VBRColor color) {
		return Pointer{Pointer::Tag::kColor, hashdag::RGB8Color{color.Get()}.GetData()};
	}
	Chunk GetLeaf(Pointer ptr) const {
		if (ptr.GetTag() != Pointer::Tag::kLeaf)
			return {};
		size_t idx = ptr.GetData() + 1;
		const size_t nm = leaves[idx], nb = leaves[idx + 1], nw = leaves[idx + 2];
		idx += 3;
		std::vector<hashdag::VBRMacroBlock> m(nm);
		std::vector<hashdag::VBRBlockHeader> b(nb);
		std::vector<uint32_t> w(nw);
		std::memcpy(m.data(), leaves.data() + idx, nm * 8);
		idx += nm * 2;
		std::memcpy(b.data(), leaves.data() + idx, nb * 8);
		idx += nb * 2;
		std::memcpy(w.data(), leaves.data() + idx, nw * 4);
		return Chunk{std::move(m), std::move(b), hashdag::VBRBitset<uint32_t, hashdag::VBRWriterContainer>{std::move(w)}};
	}
	void write_chunk(size_t idx, const Chunk &c) {
		leaves[idx++] = (uint32_t)c.GetMacroBlocks().size();
		leaves[idx++] = (uint32_t)c.GetBlockHeaders().size();
		leaves[idx++] = (uint32_t)c.GetWeightBits().GetWords().size();
		std::memcpy(leaves.data() + idx, c.GetMacroBlocks().data(), c.GetMacroBlocks().size() * 8);
		idx += c.GetMacroBlocks().size() * 2;
		std::memcpy(leaves.data() + idx, c.GetBlockHeaders().data(), c.GetBlockHeaders().size() * 8);
		idx += c.GetBlockHeaders().size() * 2;
		std::memcpy(leaves.data() + idx, c.GetWeightBits().GetWords().data(), c.GetWeightBits().GetWords().size() * 4);
	}
	Pointer SetLeaf(Pointer ptr, Chunk &&chunk) {
		const size_t data_size = chunk.GetMacroBlocks().size() * 2 + chunk.GetBlockHeaders().size() * 2 +
		                         chunk.GetWeightBits().GetWords().size() + 4;
		size_t append_size = (data_size & 1) ? data_size + 1 : data_size;
		if (!keep_history && ptr.GetTag() == Pointer::Tag::kLeaf) {
			const size_t idx = ptr.GetData(), block_size = leaves[idx];
			if (data_size <= block_size) {
				write_chunk(idx + 1, chunk);
				return ptr;
			}
			append_size = std::max(block_size << 1, append_size);
		}
		const size_t idx = leaves.size();
		leaves.resize(idx + append_size, 0u);
		leaves[idx] = (uint32_t)append_size;
		write_chunk(idx + 1, chunk);
		return Pointer{Pointer::Tag::kLeaf, (uint32_t)idx};
	}
	uint32_t GetLeafLevel() const { return leaf_level; }

	// colour of one voxel (coordinates at voxel resolution), walking the octree
	// like trace.frag:341-355 and reading leaf chunks with the reference's
	// VBRChunkIterator
	hashdag::VBRColor Fetch(Pointer root, uint32_t voxel_level, glm::u32vec3 v) const {
		Pointer p = root;
		for (uint32_t l = 0; l < leaf_level; ++l) {
			if (p.GetTag() != Pointer::Tag::kNode)
				break;
			const uint32_t s = voxel_level - 1u - l;
			p = nodes[p.GetData()][((v.x >> s) & 1u) | (((v.y >> s) & 1u) << 1u) | (((v.z >> s) & 1u) << 2u)];
		}
		if (p.GetTag() == Pointer::Tag::kColor)
			return GetFill(p);
		if (p.GetTag() != Pointer::Tag::kLeaf)
			return {};
		const uint32_t bits = voxel_level - leaf_level, m = (1u << bits) - 1u;
		uint32_t morton = 0;
		for (uint32_t b = 0; b < bits; ++b)
			morton |= (((v.x & m) >> b & 1u) << (3 * b)) | (((v.y & m) >> b & 1u) << (3 * b + 1)) |
			          (((v.z & m) >> b & 1u) << (3 * b + 2));
		hashdag::VBRChunkIterator<uint32_t, hashdag::VBRWriterContainer> it{GetLeaf(p)};
		it.Jump(morton);
		return it.GetColor();
	}
};
static_assert(hashdag::VBROctree<RefColorPool, uint32_t>);

// Colour editors of src/main.cpp:32-150 (AABBEditor, SphereEditor<kFill>,
// SphereEditor<kPaint>): the geometry of DescEditor plus the colour rules.
struct VbrDescEditor {
	DescEditor geo; // op FILL
	hashdag::VBRColor color;
	bool paint;
	hashdag::EditType EditNode(const hashdag::Config<uint32_t> &config, const hashdag::NodeCoord<uint32_t> &coord,
	                           hashdag::NodePointer<uint32_t> ptr, hashdag::VBRColor &final_color) const {
		auto edit_type = geo.EditNode(config, coord, {});
		if (geo.e.shape == HD_SHAPE_AABB) { // main.cpp:48-58
			if (edit_type == hashdag::EditType::kFill || !ptr || final_color == color)
				final_color = color;
			else
				final_color = {};
			return edit_type;
		}
		if (edit_type == hashdag::EditType::kFill) { // main.cpp:107-127
			final_color = color;
			if (paint)
				edit_type = hashdag::EditType::kNotAffected;
		} else if (!ptr || final_color == color) {
			final_color = color;
		} else
			final_color = {};
		if (paint && !ptr)
			edit_type = hashdag::EditType::kNotAffected;
		return edit_type;
	}
	bool EditVoxel(const hashdag::Config<uint32_t> &config, const hashdag::NodeCoord<uint32_t> &coord, bool voxel,
	               hashdag::VBRColor &c) const {
		const bool in_range = geo.EditVoxel(config, coord, false); // op FILL: false || in
		c = in_range || !voxel ? color : c;
		return paint ? voxel : (voxel || in_range);
	}
};

static uint32_t rd(FILE *f) {
	uint32_t v = 0;
	if (fread(&v, 4, 1, f) != 1) {
		fprintf(stderr, "short read\n");
		exit(2);
	}
	return v;
}
static void wr(FILE *f, uint32_t v) { fwrite(&v, 4, 1, f); }

template <typename HasherT>
static int run(FILE *in, FILE *out, uint32_t mode, const hashdag::Config<uint32_t> &config, const hd_config &hc) {
	uint32_t threads = rd(in), max_task_level = rd(in), n_edits = rd(in);
	std::vector<hd_edit_desc> edits(n_edits);
	if (n_edits && fread(edits.data(), sizeof(hd_edit_desc), n_edits, in) != n_edits)
		return 2;
	auto pool = std::make_unique<RefPool<HasherT>>(config, hc);
	hashdag::NodePointer<uint32_t> root{};
	std::vector<uint32_t> upsert_ptrs;
	std::vector<float> rays;
	std::vector<uint32_t> keep_at;
	std::vector<hashdag::NodePointer<uint32_t>> kept;
	std::vector<uint32_t> kept_before;
	uint64_t gc_ns = 0;
	if (mode == 4) {
		uint32_t n_keep = rd(in);
		keep_at.resize(n_keep);
		for (auto &k : keep_at)
			k = rd(in);
		kept.resize(n_keep);
	}
	RefColorPool cpool;
	RefColorPool::Pointer color_root{};
	struct VbrOp {
		uint32_t kind, colors, weight, bpw;
	};
	std::vector<VbrOp> vops;
	std::vector<uint32_t> queries;
	if (mode == 5) {
		cpool.leaf_level = rd(in);
		cpool.keep_history = rd(in) != 0;
		vops.resize(n_edits);
		for (auto &o : vops)
			o = {rd(in), rd(in), rd(in), rd(in)};
		queries.resize(3 * size_t(rd(in)));
		for (auto &q : queries)
			q = rd(in);
	}
	auto t0 = std::chrono::steady_clock::now();
	std::vector<uint64_t> edit_ns;
	if (mode == 5) {
		for (uint32_t i = 0; i < n_edits; ++i) {
			const auto te = std::chrono::steady_clock::now();
			struct Lap {
				std::vector<uint64_t> &v;
				std::chrono::steady_clock::time_point t;
				~Lap() {
					v.push_back(std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t)
					                .count());
				}
			} lap{edit_ns, te};
			if (vops[i].kind == 0) {
				root = pool->Edit(root, hashdag::StatelessEditorWrapper<uint32_t, DescEditor>{.editor = DescEditor{edits[i]}});
				continue;
			}
			hashdag::VBRColor c = vops[i].bpw == 0
			                          ? hashdag::VBRColor{hashdag::RGB8Color{vops[i].colors}}
			                          : hashdag::VBRColor{hashdag::R5G6B5Color{(uint16_t)(vops[i].colors & 0xFFFFu)},
			                                              hashdag::R5G6B5Color{(uint16_t)(vops[i].colors >> 16u)},
			                                              (uint8_t)vops[i].weight, (uint8_t)vops[i].bpw};
			hd_edit_desc g = edits[i];
			g.op = HD_OP_FILL;
			using Wrapper = hashdag::VBREditorWrapper<uint32_t, VbrDescEditor, RefColorPool>;
			auto res = pool->Edit(root,
			                      Wrapper{.editor = VbrDescEditor{DescEditor{g}, c, vops[i].kind == 2},
			                              .p_octree = &cpool,
			                              .octree_root = color_root},
			                      [](hashdag::NodePointer<uint32_t> r, auto &&state) {
				                      return std::make_pair(r, state.octree_node);
			                      });
			root = res.first;
			color_root = res.second;
		}
	} else if (mode == 4) {
		for (uint32_t i = 0; i < n_edits; ++i) {
			root = pool->Edit(root, hashdag::StatelessEditorWrapper<uint32_t, DescEditor>{.editor = DescEditor{edits[i]}});
			for (size_t k = 0; k < keep_at.size(); ++k)
				if (keep_at[k] == i)
					kept[k] = root;
		}
		for (auto &r : kept)
			kept_before.push_back(*r);
		lf::busy_pool busy(threads ? threads : 1); // one worker: the deterministic layout of the golden cases
		const auto g0 = std::chrono::steady_clock::now();
		kept = pool->ThreadedGC(&busy, kept);
		gc_ns = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - g0).count();
		root = kept.empty() ? hashdag::NodePointer<uint32_t>{} : kept.back();
	} else if (mode == 0 || mode == 3) {
		for (auto &e : edits)
			root = pool->Edit(root, hashdag::StatelessEditorWrapper<uint32_t, DescEditor>{.editor = DescEditor{e}});
	} else if (mode == 1) {
		lf::busy_pool busy(threads ? threads : 1);
		for (auto &e : edits)
			root = pool->ThreadedEdit(&busy, root, hashdag::StatelessEditorWrapper<uint32_t, DescEditor>{.editor = DescEditor{e}},
			                          max_task_level);
	} else if (mode == 2) {
		pool->make_filled_node_pointers();
		uint32_t n_ops = rd(in);
		for (uint32_t i = 0; i < n_ops; ++i) {
			uint32_t level = rd(in), len = rd(in);
			std::vector<uint32_t> w(len);
			for (auto &x : w)
				x = rd(in);
			hashdag::NodePointer<uint32_t> p;
			if (level == config.GetNodeLevels() - 1 && len == 2)
				p = pool->template upsert_leaf<false>(level, std::span<const uint32_t, 2>{w.data(), 2}, {});
			else
				p = pool->template upsert_inner_node<false>(level, std::span<const uint32_t>{w}, {});
			upsert_ptrs.push_back(*p);
		}
	}
	auto t1 = std::chrono::steady_clock::now();
	uint64_t ns = std::chrono::duration_cast<std::chrono::nanoseconds>(t1 - t0).count();

	fwrite("HDRS", 1, 4, out);
	wr(out, *root);
	wr(out, 1);
	fwrite(&ns, 8, 1, out);
	for (uint32_t l = 0; l < config.GetNodeLevels(); ++l)
		wr(out, pool->m_filled_node_pointers.empty() ? 0xFFFFFFFFu : *pool->m_filled_node_pointers[l]);
	uint32_t tb = config.GetTotalBuckets();
	wr(out, tb);
	fwrite(pool->BucketWords().data(), 4, tb, out);
	const std::vector<uint32_t> page_ids = pool->PageIds();
	wr(out, (uint32_t)page_ids.size());
	for (uint32_t i : page_ids) {
		wr(out, i);
		fwrite(pool->ReadPage(i), 4, config.GetWordsPerPage(), out);
	}
	if (mode == 4) {
		wr(out, (uint32_t)kept.size());
		for (uint32_t v : kept_before)
			wr(out, v);
		for (auto &r : kept)
			wr(out, *r);
		fwrite(&gc_ns, 8, 1, out);
	}
	if (mode == 5) {
		wr(out, color_root.pointer);
		wr(out, (uint32_t)cpool.nodes.size());
		for (auto &n : cpool.nodes)
			for (auto &p : n)
				wr(out, p.pointer);
		wr(out, (uint32_t)cpool.leaves.size());
		fwrite(cpool.leaves.data(), 4, cpool.leaves.size(), out);
		for (size_t q = 0; q + 2 < queries.size(); q += 3) {
			const hashdag::VBRColor c =
			    cpool.Fetch(color_root, config.GetVoxelLevel(), glm::u32vec3{queries[q], queries[q + 1], queries[q + 2]});
			wr(out, c.HasValue() ? 1u : 0u);
			wr(out, c.GetColors());
			wr(out, c.GetWeight());
			wr(out, c.GetBitsPerWeight());
			const glm::vec3 rgb = c.Get();
			fwrite(&rgb.x, 4, 1, out);
			fwrite(&rgb.y, 4, 1, out);
			fwrite(&rgb.z, 4, 1, out);
		}
		fwrite(edit_ns.data(), 8, edit_ns.size(), out);
	}
	if (mode == 2) {
		wr(out, (uint32_t)upsert_ptrs.size());
		fwrite(upsert_ptrs.data(), 4, upsert_ptrs.size(), out);
	}
	if (mode == 3) {
		uint32_t n = rd(in);
		std::vector<float> o(3 * size_t(n)), d(3 * size_t(n));
		if (n && (fread(o.data(), 4, o.size(), in) != o.size() || fread(d.data(), 4, d.size(), in) != d.size()))
			return 2;
		wr(out, n);
		std::vector<float> hits(4 * size_t(n));
		const auto r0 = std::chrono::steady_clock::now();
		for (uint32_t i = 0; i < n; ++i) {
			auto r = pool->template Traversal<float>(root, glm::vec3{o[3 * i], o[3 * i + 1], o[3 * i + 2]},
			                                          glm::vec3{d[3 * i], d[3 * i + 1], d[3 * i + 2]});
			hits[4 * size_t(i)] = r ? 1.f : 0.f;
			hits[4 * size_t(i) + 1] = r ? r->x : 0.f;
			hits[4 * size_t(i) + 2] = r ? r->y : 0.f;
			hits[4 * size_t(i) + 3] = r ? r->z : 0.f;
		}
		const uint64_t trace_ns =
		    std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - r0).count();
		for (uint32_t i = 0; i < n; ++i) {
			wr(out, hits[4 * size_t(i)] != 0.f ? 1u : 0u);
			fwrite(&hits[4 * size_t(i) + 1], 4, 3, out);
		}
		fwrite(&trace_ns, 8, 1, out);
	}
	return 0;
}

int main(int argc, char **argv) {
	if (argc != 3) {
		fprintf(stderr, "usage: ref_driver <request> <response>\n");
		return 2;
	}
	FILE *in = fopen(argv[1], "rb"), *out = fopen(argv[2], "wb");
	if (!in || !out)
		return 2;
	char magic[4];
	if (fread(magic, 1, 4, in) != 4 || memcmp(magic, "HDRQ", 4) != 0)
		return 2;
	uint32_t mode = rd(in);
	hashdag::Config<uint32_t> config;
	config.word_bits_per_page = rd(in);
	config.page_bits_per_bucket = rd(in);
	uint32_t L = rd(in), hasher = rd(in);
	for (uint32_t l = 0; l < L; ++l)
		config.bucket_bits_each_level.push_back(rd(in));
	if (L > HD_MAX_LEVELS || !hashdag::Config<uint32_t>::Validate(config))
		return 3;
	hd_config hc{};
	hc.word_bits_per_page = config.word_bits_per_page;
	hc.page_bits_per_bucket = config.page_bits_per_bucket;
	hc.node_levels = L;
	hc.hasher = hasher;
	for (uint32_t l = 0; l < L; ++l)
		hc.bucket_bits_each_level[l] = config.bucket_bits_each_level[l];
	int rc = hasher == HD_HASHER_ZERO ? run<ZeroHasher>(in, out, mode, config, hc)
	                                  : run<hashdag::MurmurHasher32>(in, out, mode, config, hc);
	fclose(in);
	fclose(out);
	return rc;
}
