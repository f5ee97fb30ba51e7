// hashdag_oracle.cpp -- CPU restatement of the reference HashDAG edit path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
// smoke check and the CPU-baseline leg of the benchmark call it to check or
// time the CUDA engine.  The engine itself (vkhashdag_gb300/) never links,
// loads or calls it.
//
// It restates, in plain C++, the algorithm of the reference's header library
// include/hashdag/ (AdamYuan/VkHashDAG) for the stateless sphere and box
// editors of src/main.cpp, with the same storage layout, hash functions and
// page padding rule, so that a serial edit here produces a pool that is word
// for word the pool the reference's serial NodePoolBase::Edit produces.  Each
// function names the reference lines it follows.  The threaded edit follows
// NodePoolThreadedEdit (libfork fork-join) with OpenMP tasks.
//
// Exported through a small C ABI (orc_*) for ctypes.

#include "../include/hashdag_gpu.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <bit>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <parallel/algorithm>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

using Word = uint32_t;
static constexpr Word kNull = 0xFFFFFFFFu;

// ---------------------------------------------------------------- Config
// include/hashdag/Config.hpp:15-57
struct Config {
	Word wbpp = 9, pbpb = 2, hasher = HD_HASHER_MURMUR32;
	std::vector<Word> bucket_bits;
	Word words_per_page() const { return Word(1) << wbpp; }
	Word pages_per_bucket() const { return Word(1) << pbpb; }
	Word words_per_bucket() const { return Word(1) << (wbpp + pbpb); }
	Word buckets_at(Word l) const { return Word(1) << bucket_bits[l]; }
	Word node_levels() const { return (Word)bucket_bits.size(); }
	Word voxel_level() const { return node_levels() + 1; }
	std::vector<Word> level_bases() const { // Config.hpp:33-38
		std::vector<Word> b(bucket_bits.size(), 0);
		for (size_t i = 1; i < bucket_bits.size(); ++i)
			b[i] = buckets_at(Word(i - 1)) + b[i - 1];
		return b;
	}
	uint64_t total_buckets() const {
		uint64_t t = 0;
		for (Word b : bucket_bits)
			t += uint64_t(1) << b;
		return t;
	}
	uint64_t total_pages() const { return total_buckets() << pbpb; }
};

// ---------------------------------------------------------------- hashers
// include/hashdag/Hasher.hpp:21-39 (span of any length: MurmurHash3 x86-32 body, seed 0)
static inline Word murmur_words(const Word *w, size_t n) {
	Word h = 0;
	for (size_t i = 0; i < n; ++i) {
		Word k = w[i];
		k *= 0xcc9e2d51u;
		k = (k << 15) | (k >> 17);
		k *= 0x1b873593u;
		h ^= k;
		h = (h << 13) | (h >> 19);
		h = h * 5u + 0xe6546b64u;
	}
	h ^= Word(n);
	h ^= h >> 16;
	h *= 0x85ebca6bu;
	h ^= h >> 13;
	h *= 0xc2b2ae35u;
	h ^= h >> 16;
	return h;
}
// include/hashdag/Hasher.hpp:40-48 (fixed extent 2: 64-bit finaliser, truncated)
static inline Word murmur_leaf(Word w0, Word w1) {
	uint64_t h = uint64_t(w0) | (uint64_t(w1) << 32);
	h ^= h >> 33;
	h *= 0xff51afd7ed558ccdull;
	h ^= h >> 33;
	h *= 0xc4ceb9fe1a85ec53ull;
	h ^= h >> 33;
	return Word(h);
}

// include/hashdag/NodePool.hpp:214-226 (popcount(mask)+1, 0 for an empty mask)
static inline Word inner_node_words(const Word *p) {
	Word m = *p & 0xFFu;
	return m ? Word(std::popcount(m)) + 1u : 0u;
}

// ---------------------------------------------------------------- editors
// src/main.cpp:32-150, stateless forms, restated for hd_edit_desc.
enum EditType { kNotAffected = 0, kProceed = 1, kFill = 2, kClear = 3 };

static inline EditType edit_node_type(const hd_edit_desc &e, Word voxel_level, Word level, const Word pos[3]) {
	Word bits = voxel_level - level; // NodeCoord::GetLower/UpperBoundAtLevel (NodeCoord.hpp:86-93)
	Word lb[3], ub[3];
	for (int a = 0; a < 3; ++a) {
		lb[a] = pos[a] << bits;
		ub[a] = (pos[a] + 1u) << bits;
	}
	if (e.shape == HD_SHAPE_AABB) { // AABBEditor::EditNode (src/main.cpp:36-47)
		for (int a = 0; a < 3; ++a)
			if (ub[a] <= e.p0[a] || lb[a] >= e.p1[a])
				return kNotAffected;
		bool inside = true;
		for (int a = 0; a < 3; ++a)
			inside = inside && lb[a] >= e.p0[a] && ub[a] <= e.p1[a];
		if (inside)
			return e.op == HD_OP_DIG ? kClear : kFill;
		return kProceed;
	}
	// SphereEditor::EditNode (src/main.cpp:77-106)
	int64_t lbd[3], ubd[3];
	uint64_t lb2[3], ub2[3], mx = 0;
	for (int a = 0; a < 3; ++a) {
		lbd[a] = int64_t(lb[a]) - int64_t(e.p0[a]);
		ubd[a] = int64_t(ub[a]) - int64_t(e.p0[a]);
		lb2[a] = uint64_t(lbd[a]) * uint64_t(lbd[a]);
		ub2[a] = uint64_t(ubd[a]) * uint64_t(ubd[a]);
		mx += std::max(lb2[a], ub2[a]);
	}
	if (mx <= e.r2)
		return e.op == HD_OP_DIG ? kClear : kFill;
	uint64_t mn = 0;
	for (int a = 0; a < 3; ++a) {
		if (lbd[a] > 0)
			mn += lb2[a];
		if (ubd[a] < 0)
			mn += ub2[a];
	}
	return mn > e.r2 ? kNotAffected : kProceed;
}

static inline bool voxel_in_shape(const hd_edit_desc &e, const Word p[3]) {
	if (e.shape == HD_SHAPE_AABB) // AABBEditor::VoxelInRange (src/main.cpp:55-57)
		return p[0] >= e.p0[0] && p[1] >= e.p0[1] && p[2] >= e.p0[2] && p[0] < e.p1[0] && p[1] < e.p1[1] &&
		       p[2] < e.p1[2];
	// SphereEditor::VoxelInRange (src/main.cpp:121-126)
	uint64_t n2 = 0;
	for (int a = 0; a < 3; ++a) {
		int64_t d = int64_t(p[a]) - int64_t(e.p0[a]);
		n2 += uint64_t(d) * uint64_t(d);
	}
	return n2 <= e.r2;
}
// EditVoxel (src/main.cpp:58-60 fill, :127-136 fill/dig)
static inline bool edit_voxel(const hd_edit_desc &e, const Word p[3], bool voxel) {
	bool in = voxel_in_shape(e, p);
	return e.op == HD_OP_DIG ? (voxel && !in) : (voxel || in);
}

// ---------------------------------------------------------------- pool
struct Pool {
	Config cfg;
	std::vector<Word> bases;
	std::unique_ptr<Word[]> bucket_words;
	std::vector<std::unique_ptr<Word[]>> pages;
	std::vector<Word> filled;
	std::unique_ptr<std::mutex[]> mutexes; // striped like src/DAGNodePool.hpp:43,56
	static constexpr Word kMutexes = 1024;

	explicit Pool(Config c) : cfg(std::move(c)) {
		bases = cfg.level_bases();
		bucket_words = std::make_unique<Word[]>(cfg.total_buckets());
		std::fill(bucket_words.get(), bucket_words.get() + cfg.total_buckets(), 0u);
		pages.resize(cfg.total_pages());
		mutexes = std::make_unique<std::mutex[]>(kMutexes);
	}

	// storage hooks, pattern of src/DAGNodePool.hpp:56-69
	const Word *read_page(Word page) const { return pages[page].get(); }
	Word *page_for_write(Word page) {
		if (!pages[page]) {
			pages[page] = std::make_unique<Word[]>(cfg.words_per_page()); // zero-initialised
		}
		return pages[page].get();
	}
	void write_page(Word page, Word off, const Word *w, Word n) { std::memcpy(page_for_write(page) + off, w, n * 4); }
	void zero_page(Word page, Word off, Word n) { std::memset(page_for_write(page) + off, 0, size_t(n) * 4); }

	// NodePool.hpp:75-77
	const Word *read_node(Word node) const {
		return read_page(node >> cfg.wbpp) + (node & (cfg.words_per_page() - 1u));
	}

	// NodePool.hpp:79-91
	template <bool Leaf>
	static Word find_in_span(Word base, const Word *span, Word span_len, const Word *node, Word node_len) {
		Word i = 0;
		while (node_len <= span_len - i) {
			Word w = Leaf ? 2u : inner_node_words(span + i);
			if (w == 0)
				break;
			if (w == node_len && std::equal(node, node + node_len, span + i))
				return base + i;
			i += w;
		}
		return kNull;
	}

	// NodePool.hpp:93-132
	template <bool Leaf>
	Word find_node(Word bucket, Word bucket_words_now, Word bucket_word_offset, const Word *node, Word node_len) const {
		if (bucket_words_now <= bucket_word_offset)
			return kNull;
		Word find_words = bucket_words_now - bucket_word_offset;
		Word page_index = (bucket << cfg.pbpb) | (bucket_word_offset >> cfg.wbpp);
		Word page_word_offset = bucket_word_offset & (cfg.words_per_page() - 1u);
		while (page_word_offset + find_words >= cfg.words_per_page()) {
			Word r = find_in_span<Leaf>((page_index << cfg.wbpp) | page_word_offset, read_page(page_index) + page_word_offset,
			                            cfg.words_per_page() - page_word_offset, node, node_len);
			if (r != kNull)
				return r;
			find_words -= cfg.words_per_page() - page_word_offset;
			page_word_offset = 0;
			++page_index;
		}
		if (find_words) {
			Word r = find_in_span<Leaf>((page_index << cfg.wbpp) | page_word_offset, read_page(page_index) + page_word_offset,
			                            find_words, node, node_len);
			if (r != kNull)
				return r;
		}
		return kNull;
	}

	// NodePool.hpp:134-157; returns {ptr, new_bucket_words}
	std::pair<Word, Word> append_node(Word bucket, Word bw, const Word *node, Word node_len) {
		if (uint64_t(bw) + node_len > cfg.words_per_bucket())
			return {kNull, 0};
		Word slot = bw >> cfg.wbpp;
		Word off = bw & (cfg.words_per_page() - 1u);
		Word page = (bucket << cfg.pbpb) | slot;
		if (off + node_len > cfg.words_per_page()) {
			zero_page(page, off, cfg.words_per_page() - off);
			++slot;
			++page;
			off = 0;
		}
		write_page(page, off, node, node_len);
		Word nbw = ((slot << cfg.wbpp) | off) + node_len;
		return {(page << cfg.wbpp) | off, nbw};
	}

	Word node_hash(bool leaf, const Word *node, Word len) const {
		if (cfg.hasher == HD_HASHER_ZERO)
			return 0;
		return leaf ? murmur_leaf(node[0], node[1]) : murmur_words(node, len);
	}

	// NodePool.hpp:159-212; `ok` is cleared when the bucket is full (the
	// reference silently returns fallback there; the oracle returns it too but
	// records the event).
	template <bool ThreadSafe>
	Word upsert(bool leaf, Word level, const Word *node, Word len, Word fallback, bool *ok) {
		const Word bucket = bases[level] + (node_hash(leaf, node, len) & (cfg.buckets_at(level) - 1u));
		Word &ref = bucket_words[bucket];
		if constexpr (ThreadSafe) {
			std::atomic_ref<Word> aref{ref};
			Word shared = aref.load(std::memory_order_acquire);
			Word r = leaf ? find_node<true>(bucket, shared, 0, node, len) : find_node<false>(bucket, shared, 0, node, len);
			if (r != kNull)
				return r;
			std::lock_guard<std::mutex> lk{mutexes[bucket % kMutexes]};
			Word uniq = aref.load(std::memory_order_relaxed);
			r = leaf ? find_node<true>(bucket, uniq, shared, node, len) : find_node<false>(bucket, uniq, shared, node, len);
			if (r != kNull)
				return r;
			auto [p, nbw] = append_node(bucket, uniq, node, len);
			if (p != kNull) {
				// release so that a lock-free reader that sees the new count also
				// sees the node words (the reference stores relaxed under the lock)
				aref.store(nbw, std::memory_order_release);
				return p;
			}
			if (ok)
				*ok = false;
			return fallback;
		} else {
			const Word bw = ref;
			Word r = leaf ? find_node<true>(bucket, bw, 0, node, len) : find_node<false>(bucket, bw, 0, node, len);
			if (r != kNull)
				return r;
			auto [p, nbw] = append_node(bucket, bw, node, len);
			if (p != kNull) {
				ref = nbw;
				return p;
			}
			if (ok)
				*ok = false;
			return fallback;
		}
	}

	// NodePool.hpp:240-262
	void make_filled(bool *ok) {
		if (!filled.empty())
			return;
		Word L = cfg.node_levels();
		filled.assign(L, kNull);
		Word leaf[2] = {kNull, kNull};
		filled[L - 1] = upsert<false>(true, L - 1, leaf, 2, kNull, ok);
		if (L == 1)
			return;
		for (Word l = L - 2; l != Word(-1); --l) {
			Word p = filled[l + 1];
			Word node[9] = {0xFFu, p, p, p, p, p, p, p, p};
			filled[l] = upsert<false>(false, l, node, 9, kNull, ok);
		}
	}

	// NodePoolThreadedGC.hpp:29-403 (ThreadedGC) in the order the reference runs
	// it with one worker: mark level by level from the roots (the filled root
	// first, :357-369), every bucket's node list sorted and unique (:36-37);
	// then bottom-up, leaves re-appended in place to their own bucket
	// (:223-265), inner nodes re-written with remapped children, re-hashed and
	// appended to their new bucket's cache in old-bucket / old-pointer order
	// (:105-171) and the caches flushed as the level's new bucket contents
	// (:189-213); roots remapped at level 0 (:323-328); filled pointers made
	// again (:378-381).  A bucket cache that outgrows its bucket clears `ok`
	// (the reference would write past the bucket there).
	void gc_serial(Word *roots, Word n_roots, bool *ok) {
		const Word L = cfg.node_levels(), wbpb = cfg.wbpp + cfg.pbpb, wpp = cfg.words_per_page();
		std::vector<std::vector<Word>> bucket_nodes(cfg.total_buckets());
		if (!filled.empty() && filled[0] != kNull)
			bucket_nodes[filled[0] >> wbpb].push_back(filled[0]);
		for (Word i = 0; i < n_roots; ++i)
			if (roots[i] != kNull)
				bucket_nodes[roots[i] >> wbpb].push_back(roots[i]);
		for (Word l = 0; l < L; ++l) {
			const bool leaf = l == L - 1;
			for (Word b = bases[l]; b < bases[l] + cfg.buckets_at(l); ++b) {
				std::vector<Word> &v = bucket_nodes[b];
				std::sort(v.begin(), v.end());
				v.erase(std::unique(v.begin(), v.end()), v.end());
				if (leaf)
					continue;
				for (Word node : v) {
					const Word *pn = read_node(node);
					const Word *child = pn + 1;
					for (Word m = pn[0]; m; m &= m - 1) {
						const Word c = *(child++);
						bucket_nodes[c >> wbpb].push_back(c);
					}
				}
			}
		}
		std::unordered_map<Word, Word> child_map, cur_map;
		for (Word l = L - 1; l != Word(-1); --l) {
			cur_map.clear();
			if (l == L - 1) {
				for (Word b = bases[l]; b < bases[l] + cfg.buckets_at(l); ++b) {
					Word nbw = 0;
					for (Word node : bucket_nodes[b]) {
						const Word w[2] = {read_node(node)[0], read_node(node)[1]};
						auto [np, nb] = append_node(b, nbw, w, 2);
						if (np == kNull) {
							if (ok)
								*ok = false;
							break;
						}
						cur_map[node] = np;
						nbw = nb;
					}
					bucket_words[b] = nbw;
				}
			} else {
				std::vector<std::vector<Word>> caches(cfg.buckets_at(l));
				for (Word b = bases[l]; b < bases[l] + cfg.buckets_at(l); ++b)
					for (Word node : bucket_nodes[b]) {
						const Word *pn = read_node(node);
						Word w[9];
						const Word len = inner_node_words(pn);
						std::copy(pn, pn + len, w);
						for (Word i = 1; i < len; ++i)
							w[i] = child_map.at(w[i]);
						const Word nb = bases[l] + (node_hash(false, w, len) & (cfg.buckets_at(l) - 1u));
						std::vector<Word> &cache = caches[nb - bases[l]];
						Word off = Word(cache.size());
						if ((off & (wpp - 1u)) + len > wpp)
							off = ((off >> cfg.wbpp) + 1u) << cfg.wbpp;
						cache.resize(off + len, 0u);
						std::copy(w, w + len, cache.begin() + off);
						cur_map[node] = (nb << wbpb) | off;
					}
				for (Word k = 0; k < cfg.buckets_at(l); ++k) {
					const Word b = bases[l] + k;
					const std::vector<Word> &cache = caches[k];
					if (cache.size() > cfg.words_per_bucket()) {
						if (ok)
							*ok = false;
						continue;
					}
					for (Word off = 0; off < cache.size(); off += wpp)
						write_page((b << cfg.pbpb) | (off >> cfg.wbpp), 0, cache.data() + off,
						           std::min<Word>(wpp, Word(cache.size()) - off));
					bucket_words[b] = Word(cache.size());
				}
			}
			if (l == 0)
				for (Word i = 0; i < n_roots; ++i)
					if (roots[i] != kNull)
						roots[i] = cur_map.at(roots[i]);
			std::swap(child_map, cur_map);
		}
		filled.clear();
		make_filled(ok);
	}

	// The same collection on several threads.  Each level's live nodes are a
	// bitmap over the level's pointer space (a bit per word); the sorted list of
	// live nodes (pointer order is bucket-major, so each bucket's run is its
	// sorted, unique node list) and old -> new pointers (the rank of a node's
	// bit) come from it.  Reading the live nodes' children, the per-bucket leaf
	// re-append, the remap and re-hash of inner nodes and the per-bucket layout
	// of the new caches run on all threads.  The caches take the nodes in the
	// one-worker order (a stable counting sort by new bucket of the level's
	// old-pointer order), so the pool is word for word gc_serial's; a test
	// compares the two.
	struct LiveLevel {
		Word base = 0;               // first word of the level's pointer space
		std::vector<uint64_t> bits;  // a bit per word: a live node starts there
		std::vector<Word> before;    // live nodes in the bit words before each bit word
		std::vector<Word> nodes;     // the live nodes, ascending
		std::vector<Word> fresh;     // their new pointers
		size_t rank(Word ptr) const {
			const size_t i = ptr - base;
			return before[i >> 6] + size_t(std::popcount(bits[i >> 6] & ((uint64_t(1) << (i & 63)) - 1)));
		}
		void set(Word ptr) {
			const size_t i = ptr - base;
			std::atomic_ref<uint64_t>(bits[i >> 6]).fetch_or(uint64_t(1) << (i & 63), std::memory_order_relaxed);
		}
		void build_list(int threads) { // before[] and nodes[] from bits[]
			const size_t nw = bits.size();
			before.assign(nw + 1, 0);
			const size_t parts = size_t(std::max(1, threads)) * 4, per = (nw + parts - 1) / parts;
			std::vector<size_t> part_count(parts + 1, 0);
#pragma omp parallel for num_threads(threads) schedule(static, 1)
			for (size_t k = 0; k < parts; ++k) {
				size_t c = 0;
				for (size_t w = k * per; w < std::min(nw, (k + 1) * per); ++w)
					c += size_t(std::popcount(bits[w]));
				part_count[k + 1] = c;
			}
			for (size_t k = 0; k < parts; ++k)
				part_count[k + 1] += part_count[k];
			nodes.resize(part_count[parts]);
#pragma omp parallel for num_threads(threads) schedule(static, 1)
			for (size_t k = 0; k < parts; ++k) {
				size_t c = part_count[k];
				for (size_t w = k * per; w < std::min(nw, (k + 1) * per); ++w) {
					before[w] = Word(c);
					for (uint64_t m = bits[w]; m; m &= m - 1)
						nodes[c++] = base + Word(w * 64 + size_t(std::countr_zero(m)));
				}
			}
			before[nw] = Word(part_count[parts]);
		}
	};
	void gc(Word *roots, Word n_roots, bool *ok, int threads) {
		const Word L = cfg.node_levels(), wbpb = cfg.wbpp + cfg.pbpb, wpp = cfg.words_per_page();
		if (threads < 1)
			threads = omp_get_max_threads();
		std::vector<LiveLevel> lv(L);
		for (Word l = 0; l < L; ++l) {
			lv[l].base = bases[l] << wbpb;
			lv[l].bits.assign(((size_t(cfg.buckets_at(l)) << wbpb) + 63) / 64, 0);
		}
		if (!filled.empty() && filled[0] != kNull)
			lv[0].set(filled[0]);
		for (Word i = 0; i < n_roots; ++i)
			if (roots[i] != kNull)
				lv[0].set(roots[i]);
		for (Word l = 0; l < L; ++l) { // mark: the children of the live nodes of level l
			lv[l].build_list(threads);
			if (l + 1 == L)
				break;
			const std::vector<Word> &cur = lv[l].nodes;
			LiveLevel &nxt = lv[l + 1];
#pragma omp parallel for num_threads(threads) schedule(static)
			for (size_t i = 0; i < cur.size(); ++i) {
				const Word *pn = read_node(cur[i]);
				const Word n = Word(std::popcount(pn[0] & 0xFFu));
				for (Word j = 1; j <= n; ++j)
					nxt.set(pn[j]);
			}
		}
		std::atomic<bool> all_ok{true};
		for (Word l = L - 1; l != Word(-1); --l) {
			LiveLevel &me = lv[l];
			const std::vector<Word> &cur = me.nodes;
			me.fresh.assign(cur.size(), kNull);
			const Word b0 = bases[l], nb_count = cfg.buckets_at(l);
			if (l == L - 1) { // leaves re-appended to their own bucket in pointer order
				std::vector<size_t> run(size_t(nb_count) + 1, 0); // each bucket's run of the sorted list
				for (Word p : cur)
					++run[(p >> wbpb) - b0 + 1];
				for (Word k = 0; k < nb_count; ++k)
					run[k + 1] += run[k];
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64)
				for (Word k = 0; k < nb_count; ++k) {
					const Word b = b0 + k;
					Word nbw = 0;
					for (size_t i = run[k]; i < run[k + 1]; ++i) {
						const Word *pn = read_node(cur[i]);
						const Word w[2] = {pn[0], pn[1]};
						auto [np, nb] = append_node(b, nbw, w, 2);
						if (np == kNull) {
							all_ok = false;
							break;
						}
						me.fresh[i] = np;
						nbw = nb;
					}
					bucket_words[b] = nbw;
				}
			} else {
				// remapped words and new bucket of every live node
				const LiveLevel &below = lv[l + 1];
				std::vector<std::array<Word, 9>> words(cur.size());
				std::vector<Word> len(cur.size()), nbk(cur.size());
#pragma omp parallel for num_threads(threads) schedule(static)
				for (size_t i = 0; i < cur.size(); ++i) {
					const Word *pn = read_node(cur[i]);
					const Word n = inner_node_words(pn);
					words[i][0] = pn[0];
					for (Word j = 1; j < n; ++j)
						words[i][j] = below.fresh[below.rank(pn[j])];
					len[i] = n;
					nbk[i] = node_hash(false, words[i].data(), n) & (nb_count - 1u);
				}
				// stable counting sort by new bucket: a bucket's cache in old-pointer order
				std::vector<size_t> start(size_t(nb_count) + 1, 0), order(cur.size());
				for (size_t i = 0; i < cur.size(); ++i)
					++start[nbk[i] + 1];
				for (Word k = 0; k < nb_count; ++k)
					start[k + 1] += start[k];
				{
					std::vector<size_t> fill(start.begin(), start.end() - 1);
					for (size_t i = 0; i < cur.size(); ++i)
						order[fill[nbk[i]]++] = i;
				}
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64)
				for (Word k = 0; k < nb_count; ++k) {
					const Word b = b0 + k;
					std::vector<Word> cache;
					for (size_t j = start[k]; j < start[k + 1]; ++j) {
						const size_t i = order[j];
						Word off = Word(cache.size());
						if ((off & (wpp - 1u)) + len[i] > wpp)
							off = ((off >> cfg.wbpp) + 1u) << cfg.wbpp;
						cache.resize(off + len[i], 0u);
						std::copy(words[i].begin(), words[i].begin() + len[i], cache.begin() + off);
						me.fresh[i] = (b << wbpb) | off;
					}
					if (cache.size() > cfg.words_per_bucket()) {
						all_ok = false;
						continue;
					}
					for (Word off = 0; off < cache.size(); off += wpp)
						write_page((b << cfg.pbpb) | (off >> cfg.wbpp), 0, cache.data() + off,
						           std::min<Word>(wpp, Word(cache.size()) - off));
					bucket_words[b] = Word(cache.size());
				}
			}
			if (l == 0)
				for (Word i = 0; i < n_roots; ++i)
					if (roots[i] != kNull)
						roots[i] = me.fresh[me.rank(roots[i])];
			if (l + 1 < L)
				lv[l + 1] = LiveLevel{}; // the level below is no longer needed
		}
		if (!all_ok && ok)
			*ok = false;
		filled.clear();
		make_filled(ok);
	}

	// NodePool.hpp:278-309
	std::array<Word, 9> unpack(Word ptr) const {
		std::array<Word, 9> u;
		u.fill(kNull);
		u[0] = 0;
		if (ptr == kNull)
			return u;
		const Word *p = read_node(ptr);
		Word mask = p[0];
		u[0] = mask;
		const Word *nx = p + 1;
		for (Word m = mask & 0xFFu; m; m &= m - 1)
			u[1 + std::countr_zero(m)] = *nx++;
		return u;
	}
	// NodePool.hpp:272-277
	static Word pack_inplace(std::array<Word, 9> &u) {
		Word mask = u[0], *c = u.data() + 1, *nx = c;
		for (Word m = mask & 0xFFu; m; m &= m - 1)
			*nx++ = c[std::countr_zero(m)];
		return Word(nx - u.data());
	}

	// NodePool.hpp:319-343 with NodeCoord::GetLeafCoord (NodeCoord.hpp:32-43)
	template <bool ThreadSafe>
	Word edit_leaf(const hd_edit_desc &e, Word leaf_ptr, Word level, const Word pos[3], bool *ok) {
		Word leaf[2] = {0, 0};
		if (leaf_ptr != kNull) {
			const Word *p = read_node(leaf_ptr);
			leaf[0] = p[0];
			leaf[1] = p[1];
		}
		bool changed = false;
		for (Word i = 0; i < 64; ++i) {
			Word vp[3] = {(pos[0] << 2) | ((i >> 2) & 2u) | (i & 1u), (pos[1] << 2) | ((i >> 3) & 2u) | ((i >> 1) & 1u),
			              (pos[2] << 2) | ((i >> 4) & 2u) | ((i >> 2) & 1u)};
			bool v = (leaf[i >> 5] >> (i & 31)) & 1u;
			bool nv = edit_voxel(e, vp, v);
			changed |= nv != v;
			leaf[i >> 5] ^= Word(nv != v) << (i & 31);
		}
		if (!changed)
			return leaf_ptr;
		if (leaf[0] == 0 && leaf[1] == 0)
			return kNull;
		return upsert<ThreadSafe>(true, level, leaf, 2, leaf_ptr, ok);
	}

	// NodePool.hpp:345-360 (terminal part); returns true if the child must be recursed
	bool edit_switch(const hd_edit_desc &e, Word ptr, Word level, const Word pos[3], Word *out) const {
		EditType t = edit_node_type(e, cfg.voxel_level(), level, pos);
		if (t == kClear) {
			*out = kNull;
			return false;
		}
		if (t == kFill) {
			*out = filled[level];
			return false;
		}
		if (t == kNotAffected) {
			*out = ptr;
			return false;
		}
		return true;
	}

	static void child_pos(const Word pos[3], Word c, Word out[3]) { // NodeCoord.hpp:18-28
		out[0] = (pos[0] << 1) | (c & 1u);
		out[1] = (pos[1] << 1) | ((c >> 1) & 1u);
		out[2] = (pos[2] << 1) | ((c >> 2) & 1u);
	}

	// NodePool.hpp:362-396
	template <bool ThreadSafe>
	Word edit_node(const hd_edit_desc &e, Word ptr, Word level, const Word pos[3], bool *ok) {
		if (level == cfg.node_levels() - 1)
			return edit_leaf<ThreadSafe>(e, ptr, level, pos, ok);
		std::array<Word, 9> u = unpack(ptr);
		bool changed = false;
		for (Word i = 0; i < 8; ++i) {
			Word cp[3];
			child_pos(pos, i, cp);
			Word old = u[1 + i], nw;
			if (edit_switch(e, old, level + 1, cp, &nw))
				nw = edit_node<ThreadSafe>(e, old, level + 1, cp, ok);
			changed |= nw != old;
			u[1 + i] = nw;
			u[0] ^= Word((nw != kNull) != (old != kNull)) << i;
		}
		if (!changed)
			return ptr;
		if (!u[0])
			return kNull;
		Word len = pack_inplace(u);
		return upsert<ThreadSafe>(false, level, u.data(), len, ptr, ok);
	}

	// NodePool.hpp:405-417
	Word edit(Word root, const hd_edit_desc &e, bool *ok) {
		make_filled(ok);
		Word zero[3] = {0, 0, 0}, out;
		if (!edit_switch(e, root, 0, zero, &out))
			return out;
		return edit_node<false>(e, root, 0, zero, ok);
	}

	// NodePoolThreadedEdit.hpp:27-99 (lf_edit_node), fork-join with OpenMP tasks
	Word t_edit_node(const hd_edit_desc &e, Word ptr, Word level, const Word pos[3], Word max_task_level, bool *ok) {
		if (level == cfg.node_levels() - 1)
			return edit_leaf<true>(e, ptr, level, pos, ok);
		if (level >= max_task_level)
			return edit_node<true>(e, ptr, level, pos, ok);
		std::array<Word, 9> u = unpack(ptr);
		Word nc[8];
		Word cps[8][3];
		bool fork[8];
		for (Word i = 0; i < 8; ++i) {
			child_pos(pos, i, cps[i]);
			fork[i] = edit_switch(e, u[1 + i], level + 1, cps[i], &nc[i]);
		}
		// every forked child but the last becomes a task, the last runs on this
		// thread (NodePoolThreadedEdit.hpp:58-74: .fork() except for the last)
		Word last = 8;
		for (Word i = 0; i < 8; ++i)
			if (fork[i])
				last = i;
		for (Word i = 0; i < last; ++i) {
			if (!fork[i])
				continue;
#pragma omp task default(none) firstprivate(i, level, max_task_level) shared(e, u, nc, cps, ok)
			nc[i] = t_edit_node(e, u[1 + i], level + 1, cps[i], max_task_level, ok);
		}
		if (last < 8)
			nc[last] = t_edit_node(e, u[1 + last], level + 1, cps[last], max_task_level, ok);
#pragma omp taskwait
		bool changed = false;
		for (Word i = 0; i < 8; ++i) {
			Word old = u[1 + i];
			changed |= nc[i] != old;
			u[0] ^= Word((nc[i] != kNull) != (old != kNull)) << i;
			u[1 + i] = nc[i];
		}
		if (!changed)
			return ptr;
		if (!u[0])
			return kNull;
		Word len = pack_inplace(u);
		return upsert<true>(false, level, u.data(), len, ptr, ok);
	}

	// NodePoolThreadedEdit.hpp:104-126, called by one thread of a running team
	Word threaded_edit_in_team(Word root, const hd_edit_desc &e, Word max_task_level, bool *ok) {
		Word zero[3] = {0, 0, 0}, out;
		if (!edit_switch(e, root, 0, zero, &out))
			return out;
		return t_edit_node(e, root, 0, zero, max_task_level, ok);
	}
	// ThreadedEdit of each edit in turn on one thread team that lives across
	// the edits, as the application's lf::busy_pool does (src/main.cpp:159,
	// busy_pool.hpp:117-145): the other threads wait in the team for the
	// tasks of the next edit instead of being woken per edit.
	Word threaded_edits(Word root, const hd_edit_desc *e, Word n, Word max_task_level, int threads, bool *ok) {
		make_filled(ok);
		Word r = root;
#pragma omp parallel num_threads(threads) default(none) shared(r, e, n, max_task_level, ok)
		{
#pragma omp single
			for (Word i = 0; i < n; ++i)
				r = threaded_edit_in_team(r, e[i], max_task_level, ok);
		}
		return r;
	}

	// occupancy of one voxel
	bool query(Word root, const Word v[3]) const {
		Word L = cfg.node_levels(), ptr = root;
		if (ptr == kNull)
			return false;
		for (Word l = 0; l + 1 < L; ++l) {
			Word sh = cfg.voxel_level() - l - 1;
			Word c = ((v[0] >> sh) & 1u) | (((v[1] >> sh) & 1u) << 1) | (((v[2] >> sh) & 1u) << 2);
			const Word *p = read_node(ptr);
			Word mask = p[0] & 0xFFu;
			if (!((mask >> c) & 1u))
				return false;
			ptr = p[1 + std::popcount(mask & ((1u << c) - 1u))];
			if (ptr == kNull)
				return false;
		}
		const Word *p = read_node(ptr);
		Word i = ((v[0] >> 1) & 1u) << 3 | ((v[1] >> 1) & 1u) << 4 | ((v[2] >> 1) & 1u) << 5 | (v[0] & 1u) |
		         (v[1] & 1u) << 1 | (v[2] & 1u) << 2;
		return (p[i >> 5] >> (i & 31)) & 1u;
	}
};

// ---------------------------------------------------------------- canonical DAG
// Canonical form of the reachable DAG: per level, the sorted set of node tuples
// whose child pointers are replaced by the child's rank in the sorted tuple
// list of the level below.  Equal canonical forms <=> equal voxel occupancy.
static inline uint64_t mix64(uint64_t x) {
	x ^= x >> 30;
	x *= 0xbf58476d1ce4e5b9ull;
	x ^= x >> 27;
	x *= 0x94d049bb133111ebull;
	x ^= x >> 31;
	return x;
}

struct Canon {
	std::vector<uint64_t> counts, digests;
	bool ok = true;
	int bad_level = -1; // first level holding an invalid pointer
};

// A pointer names a node of `level` if it lies below its bucket's word count,
// in a bucket of that level, on a page that exists.
static bool valid_ptr(const Pool &pool, Word ptr, Word level) {
	const Word wbb = pool.cfg.wbpp + pool.cfg.pbpb;
	const uint64_t bucket = ptr >> wbb;
	if (bucket < pool.bases[level] || bucket >= uint64_t(pool.bases[level]) + pool.cfg.buckets_at(level))
		return false;
	if ((ptr & ((Word(1) << wbb) - 1u)) >= pool.bucket_words[bucket])
		return false;
	return (ptr >> pool.cfg.wbpp) < pool.pages.size() && pool.pages[ptr >> pool.cfg.wbpp] != nullptr;
}

static Canon canonical_simple(const Pool &pool, Word root) {
	Word L = pool.cfg.node_levels();
	Canon c;
	c.counts.assign(L, 0);
	c.digests.assign(L, 0);
	if (root == kNull)
		return c;
	if (!valid_ptr(pool, root, 0)) {
		c.ok = false;
		c.bad_level = 0;
		return c;
	}
	// reachable node pointers per level
	std::vector<std::vector<Word>> lv(L);
	lv[0].push_back(root);
	for (Word l = 0; l + 1 < L; ++l) {
		std::unordered_set<Word> seen;
		for (Word p : lv[l]) {
			const Word *n = pool.read_node(p);
			Word k = std::popcount(n[0] & 0xFFu);
			for (Word j = 0; j < k; ++j) {
				if (!valid_ptr(pool, n[1 + j], l + 1)) {
					c.ok = false;
					c.bad_level = l + 1;
					return c;
				}
				if (seen.insert(n[1 + j]).second)
					lv[l + 1].push_back(n[1 + j]);
			}
		}
	}
	std::unordered_map<Word, Word> rank_below, rank_here;
	for (Word l = L; l-- > 0;) {
		std::vector<std::vector<Word>> tuples;
		tuples.reserve(lv[l].size());
		for (Word p : lv[l]) {
			const Word *n = pool.read_node(p);
			std::vector<Word> t;
			if (l == L - 1) {
				t = {n[0], n[1]};
			} else {
				Word k = std::popcount(n[0] & 0xFFu);
				t.push_back(n[0]);
				for (Word j = 0; j < k; ++j) {
					auto it = rank_below.find(n[1 + j]);
					if (it == rank_below.end()) {
						c.ok = false;
						t.push_back(kNull);
					} else
						t.push_back(it->second);
				}
			}
			tuples.push_back(std::move(t));
		}
		std::vector<Word> order(tuples.size());
		for (Word i = 0; i < order.size(); ++i)
			order[i] = i;
		std::sort(order.begin(), order.end(), [&](Word a, Word b) { return tuples[a] < tuples[b]; });
		rank_here.clear();
		uint64_t d = 0x6a09e667f3bcc909ull ^ l;
		Word rank = 0;
		for (Word i = 0; i < order.size(); ++i) {
			if (i > 0 && tuples[order[i]] == tuples[order[i - 1]]) {
				c.ok = false; // duplicate content at one level: the DAG is not reduced
			} else if (i > 0)
				++rank;
			rank_here[lv[l][order[i]]] = rank;
			if (i == 0 || tuples[order[i]] != tuples[order[i - 1]]) {
				d = mix64(d ^ tuples[order[i]].size());
				for (Word w : tuples[order[i]])
					d = mix64(d ^ w);
			}
		}
		c.counts[l] = tuples.empty() ? 0 : rank + 1;
		c.digests[l] = d;
		rank_below.swap(rank_here);
	}
	return c;
}

// The same canonical form for large DAGs (10^8 nodes): the reachable
// pointers of a level are a sorted array (children gathered on all threads,
// then sorted and made unique), a child's rank is a binary search in the
// level below, and the tuples of a level are sorted on all threads.  Tuples
// are compared word by word with zero padding and then by length, which is the
// order std::vector<Word> gives (a prefix sorts first), so counts and digests
// equal canonical_simple's.
struct CanonTuple {
	Word w[9];
	Word len;
	Word idx; // position in the level's sorted pointer array
};
static bool tuple_less(const CanonTuple &a, const CanonTuple &b) {
	for (int k = 0; k < 9; ++k)
		if (a.w[k] != b.w[k])
			return a.w[k] < b.w[k];
	return a.len < b.len;
}
static bool tuple_same(const CanonTuple &a, const CanonTuple &b) {
	if (a.len != b.len)
		return false;
	for (Word k = 0; k < a.len; ++k)
		if (a.w[k] != b.w[k])
			return false;
	return true;
}

static Canon canonical(const Pool &pool, Word root) {
	const Word L = pool.cfg.node_levels();
	Canon c;
	c.counts.assign(L, 0);
	c.digests.assign(L, 0);
	if (root == kNull)
		return c;
	if (!valid_ptr(pool, root, 0)) {
		c.ok = false;
		c.bad_level = 0;
		return c;
	}
	std::vector<std::vector<Word>> lv(L);
	lv[0].push_back(root);
	for (Word l = 0; l + 1 < L; ++l) {
		const std::vector<Word> &cur = lv[l];
		std::vector<Word> kids;
		std::atomic<int> bad{0};
#pragma omp parallel
		{
			std::vector<Word> mine;
#pragma omp for schedule(static) nowait
			for (int64_t i = 0; i < int64_t(cur.size()); ++i) {
				const Word *n = pool.read_node(cur[i]);
				const Word k = std::popcount(n[0] & 0xFFu);
				for (Word j = 0; j < k; ++j) {
					if (!valid_ptr(pool, n[1 + j], l + 1))
						bad = 1;
					else
						mine.push_back(n[1 + j]);
				}
			}
#pragma omp critical
			kids.insert(kids.end(), mine.begin(), mine.end());
		}
		if (bad) {
			c.ok = false;
			c.bad_level = int(l + 1);
			return c;
		}
		__gnu_parallel::sort(kids.begin(), kids.end());
		kids.erase(std::unique(kids.begin(), kids.end()), kids.end());
		lv[l + 1].swap(kids);
	}
	std::vector<Word> rank_below, rank_here;
	for (Word l = L; l-- > 0;) {
		const std::vector<Word> &ptrs = lv[l];
		const std::vector<Word> &below = l + 1 < L ? lv[l + 1] : ptrs;
		std::vector<CanonTuple> t(ptrs.size());
		std::atomic<int> missing{0};
#pragma omp parallel for schedule(static)
		for (int64_t i = 0; i < int64_t(ptrs.size()); ++i) {
			CanonTuple &x = t[i];
			std::fill(x.w, x.w + 9, 0u);
			x.idx = Word(i);
			const Word *n = pool.read_node(ptrs[i]);
			if (l == L - 1) {
				x.w[0] = n[0];
				x.w[1] = n[1];
				x.len = 2;
				continue;
			}
			const Word k = std::popcount(n[0] & 0xFFu);
			x.w[0] = n[0];
			x.len = k + 1;
			for (Word j = 0; j < k; ++j) {
				auto it = std::lower_bound(below.begin(), below.end(), n[1 + j]);
				if (it == below.end() || *it != n[1 + j]) {
					missing = 1;
					x.w[1 + j] = kNull;
				} else
					x.w[1 + j] = rank_below[it - below.begin()];
			}
		}
		if (missing)
			c.ok = false;
		__gnu_parallel::sort(t.begin(), t.end(), tuple_less);
		rank_here.assign(ptrs.size(), 0);
		uint64_t d = 0x6a09e667f3bcc909ull ^ l;
		Word rank = 0;
		for (size_t i = 0; i < t.size(); ++i) {
			const bool same = i > 0 && tuple_same(t[i], t[i - 1]);
			if (same)
				c.ok = false; // duplicate content at one level: the DAG is not reduced
			else if (i > 0)
				++rank;
			rank_here[t[i].idx] = rank;
			if (!same) {
				d = mix64(d ^ t[i].len);
				for (Word k = 0; k < t[i].len; ++k)
					d = mix64(d ^ t[i].w[k]);
			}
		}
		c.counts[l] = t.empty() ? 0 : rank + 1;
		c.digests[l] = d;
		rank_below.swap(rank_here);
	}
	return c;
}

// ---------------------------------------------------------------- ray traversal
// NodePoolTraversal::Traversal<float> (include/hashdag/NodePoolTraversal.hpp:93-256)
// extended with the voxel position / size output of shader/src/trace.frag:223-246.
// Compiled with -ffp-contract=off so every float operation rounds like the GPU
// kernel built with -fmad=false.
static inline Word f2w(float f) {
	Word w;
	std::memcpy(&w, &f, 4);
	return w;
}
static inline float w2f(Word w) {
	float f;
	std::memcpy(&f, &w, 4);
	return f;
}
static inline int find_msb(Word x) { return x ? 31 - std::countl_zero(x) : -1; }
// glm::abs for float (x >= 0 ? x : -x)
static inline float abs_ref(float x) { return x >= 0.0f ? x : -x; }

// Lod: the level-of-detail cut of shader/src/trace.frag:148 / beam.frag:128;
// *scale_out = size of the cube the ray stopped in (beam.frag:203).
template <bool Lod>
static hd_hit trace_ray_core(const Pool &pool, Word root, const float o_in[3], const float d_in[3], float proj_factor,
                             float proj_bias, float *scale_out) {
	hd_hit out{};
	out.hit = 0;
	if (root == kNull)
		return out;
	constexpr int kStack = 23;
	const float eps = w2f((127u - 23u) << 23); // exp2(-23) == FLT_EPSILON
	Word stack[kStack];
	for (int k = 0; k < kStack; ++k) // every entry holds a node pointer before the first push
		stack[k] = root;
	float o[3] = {o_in[0] + 1.0f, o_in[1] + 1.0f, o_in[2] + 1.0f};
	float d[3];
	for (int a = 0; a < 3; ++a)
		d[a] = abs_ref(d_in[a]) > eps ? d_in[a] : (d_in[a] >= 0 ? eps : -eps);
	float tc[3], tb[3];
	for (int a = 0; a < 3; ++a) {
		tc[a] = 1.0f / -abs_ref(d[a]);
		tb[a] = tc[a] * o[a];
	}
	Word octant = 0;
	for (int a = 0; a < 3; ++a)
		if (d[a] > 0.0f)
			octant ^= 1u << a, tb[a] = 3.0f * tc[a] - tb[a];
	float t_min = std::max(std::max(2.0f * tc[0] - tb[0], 2.0f * tc[1] - tb[1]), 2.0f * tc[2] - tb[2]);
	float t_max = std::min(std::min(tc[0] - tb[0], tc[1] - tb[1]), tc[2] - tb[2]);
	float h = t_max;
	t_min = std::max(t_min, 0.0f);
	t_max = std::min(t_max, 1.0f);
	Word parent = root, child_bits = 0;
	float pos[3] = {1.0f, 1.0f, 1.0f};
	Word idx = 0;
	for (int a = 0; a < 3; ++a)
		if (1.5f * tc[a] - tb[a] > t_min)
			idx ^= 1u << a, pos[a] = 1.5f;
	int scale = kStack - 1;
	float scale_exp2 = 0.5f;
	const Word leaf_level = pool.cfg.node_levels();
	const int leaf_scale = kStack - int(leaf_level);
	for (;;) {
		if (child_bits == 0u) {
			if (scale > leaf_scale)
				child_bits = pool.read_node(parent)[0];
			else if (scale == leaf_scale) {
				const Word *p = pool.read_node(parent);
				Word l0 = p[0], l1 = p[1];
				child_bits = ((l0 & 0xFFu) ? 1u : 0u) | ((l0 & 0xFF00u) ? 2u : 0u) | ((l0 & 0xFF0000u) ? 4u : 0u) |
				             ((l0 & 0xFF000000u) ? 8u : 0u) | ((l1 & 0xFFu) ? 16u : 0u) | ((l1 & 0xFF00u) ? 32u : 0u) |
				             ((l1 & 0xFF0000u) ? 64u : 0u) | ((l1 & 0xFF000000u) ? 128u : 0u);
			} else
				child_bits = parent;
		}
		float tcorner[3] = {pos[0] * tc[0] - tb[0], pos[1] * tc[1] - tb[1], pos[2] * tc[2] - tb[2]};
		float tc_max = std::min(std::min(tcorner[0], tcorner[1]), tcorner[2]);
		Word child_shift = idx ^ octant;
		Word child_mask = 1u << child_shift;
		if ((child_bits & child_mask) != 0 && t_min <= t_max) {
			float half = scale_exp2 * 0.5f;
			float tcen[3] = {half * tc[0] + tcorner[0], half * tc[1] + tcorner[1], half * tc[2] + tcorner[2]};
			if (scale < leaf_scale || (Lod && scale_exp2 * proj_factor < tc_max + proj_bias))
				break;
			if (tc_max < h)
				stack[scale] = parent;
			h = tc_max;
			if (scale > leaf_scale)
				parent = pool.read_node(parent + 1u + std::popcount(child_bits & (child_mask - 1u)))[0];
			else
				parent = (pool.read_node(parent + (child_shift >> 2u))[0] >> ((child_shift & 3u) << 3u)) & 0xFFu;
			idx = 0;
			--scale;
			scale_exp2 = half;
			for (int a = 0; a < 3; ++a)
				if (tcen[a] > t_min)
					idx ^= 1u << a, pos[a] += scale_exp2;
			child_bits = 0;
			continue;
		}
		Word step = 0;
		for (int a = 0; a < 3; ++a)
			if (tcorner[a] <= tc_max)
				step ^= 1u << a, pos[a] -= scale_exp2;
		t_min = tc_max;
		idx ^= step;
		if ((idx & step) != 0) {
			Word diff = 0;
			for (int a = 0; a < 3; ++a)
				if (step & (1u << a))
					diff |= f2w(pos[a]) ^ f2w(pos[a] + scale_exp2);
			scale = find_msb(diff);
			if (scale >= kStack || scale < 0) {
				scale = kStack;
				break;
			}
			scale_exp2 = w2f(Word(scale - kStack + 127) << 23);
			parent = stack[scale];
			Word sh[3];
			for (int a = 0; a < 3; ++a) {
				sh[a] = f2w(pos[a]) >> scale;
				pos[a] = w2f(sh[a] << scale);
			}
			idx = (sh[0] & 1u) | ((sh[1] & 1u) << 1) | ((sh[2] & 1u) << 2);
			h = 0.0f;
			child_bits = 0;
		}
	}
	bool hit = scale < kStack && t_min <= t_max;
	if (scale_out)
		*scale_out = scale_exp2;
	out.hit = hit ? 1u : 0u;
	out.t = t_min;
	const Word voxel_level = leaf_level + 1u;
	const int voxel_scale = kStack - int(voxel_level);
	if (hit) {
		Word size = 1u << (scale - voxel_scale);
		for (int a = 0; a < 3; ++a) {
			Word vp = (f2w(pos[a]) & 0x7FFFFFu) >> voxel_scale;
			if (octant & (1u << a))
				vp = (1u << voxel_level) - size - vp;
			out.voxel[a] = vp;
		}
		out.size = size;
		out.level = voxel_level - Word(find_msb(size));
		for (int a = 0; a < 3; ++a) {
			float p = pos[a];
			if (octant & (1u << a))
				p = 3.0f - scale_exp2 - p;
			float q = o[a] + t_min * d[a];
			q = std::min(std::max(q, p), p + scale_exp2);
			out.pos[a] = q - 1.0f;
		}
	}
	return out;
}

static hd_hit trace_ray(const Pool &pool, Word root, const float o_in[3], const float d_in[3]) {
	return trace_ray_core<false>(pool, root, o_in, d_in, 0.0f, 0.0f, nullptr);
}

// Camera_GenRay (shader/src/trace.frag:366-370) at the centre of pixel (px, py) of a w x h image.
static void pinhole_dir(const hd_camera &cam, Word px, Word py, Word w, Word h, float d[3]) {
	const float u = ((float(px) + 0.5f) / float(w)) * 2.0f - 1.0f;
	const float v = ((float(py) + 0.5f) / float(h)) * 2.0f - 1.0f;
	float dd[3];
	for (int a = 0; a < 3; ++a)
		dd[a] = (cam.look[a] - cam.side[a] * u) - cam.up[a] * v;
	const float len2 = (dd[0] * dd[0] + dd[1] * dd[1]) + dd[2] * dd[2];
	const float inv = 1.0f / std::sqrt(len2);
	for (int a = 0; a < 3; ++a)
		d[a] = dd[a] * inv;
}

static int floor_div(long long a, long long b) { return int(a >= 0 ? a / b : -((-a + b - 1) / b)); }

// beam.frag main over every 8x8 block, then trace.frag main with
// BEAM_OPTIMIZATION (beam_proj <= 0: without the prepass).  Pixels are
// camera-major, row-major, like the device.
static void trace_pinhole_lod(const Pool &pool, Word root, const hd_camera *cams, Word n_cams, Word w, Word h,
                              float proj, float beam_proj, hd_hit *out, int threads) {
	const Word bw = (w + 7) / 8, bh = (h + 7) / 8;
	const bool use_beam = beam_proj > 0.0f;
	std::vector<float> beam(use_beam ? size_t(n_cams) * bw * bh : 0);
	const float inf = w2f(0x7F800000u);
	if (use_beam) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
		for (int64_t i = 0; i < int64_t(beam.size()); ++i) {
			const Word c = Word(i / (int64_t(bw) * bh)), r = Word(i % (int64_t(bw) * bh));
			float d[3];
			pinhole_dir(cams[c], r % bw, r / bw, bw, bh, d);
			float sexp = 0.0f;
			const hd_hit hh = trace_ray_core<true>(pool, root, cams[c].position, d, beam_proj, 0.0f, &sexp);
			beam[size_t(i)] = hh.hit ? std::max(hh.t - sexp, 0.0f) : inf;
		}
	}
	const int64_t per = int64_t(w) * h, total = per * n_cams;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 4096)
	for (int64_t i = 0; i < total; ++i) {
		const Word c = Word(i / per), px = Word(i % per % w), py = Word(i % per / w);
		float d[3], o[3] = {cams[c].position[0], cams[c].position[1], cams[c].position[2]};
		pinhole_dir(cams[c], px, py, w, h, d);
		float bias = 0.0f;
		if (use_beam) {
			const float *b = beam.data() + size_t(c) * bw * bh;
			const int i0 = floor_div((2ll * px + 1) * bw - w, 2ll * w), j0 = floor_div((2ll * py + 1) * bh - h, 2ll * h);
			const int xs[2] = {std::clamp(i0, 0, int(bw) - 1), std::clamp(i0 + 1, 0, int(bw) - 1)};
			const int ys[2] = {std::clamp(j0, 0, int(bh) - 1), std::clamp(j0 + 1, 0, int(bh) - 1)};
			float m = b[size_t(ys[0]) * bw + xs[0]];
			for (int k = 1; k < 4; ++k)
				m = std::min(m, b[size_t(ys[k >> 1]) * bw + xs[k & 1]]);
			bias = m * 0.98f;
			if (f2w(bias) == 0x7F800000u) { // the block's ray missed
				out[i] = hd_hit{};
				continue;
			}
			for (int a = 0; a < 3; ++a)
				o[a] = o[a] + bias * d[a];
		}
		out[i] = trace_ray_core<true>(pool, root, o, d, proj, bias, nullptr);
	}
}

// ---------------------------------------------------------------- VBR colour
// Colour editing through VBREditorWrapper (include/hashdag/VBREditor.hpp:26-107)
// into the application's colour octree (src/DAGColorPool.hpp:20-218) with VBR
// leaf chunks (include/hashdag/VBRColor.hpp:222-491), and the colour lookup of
// trace.frag:272-356.
//
// Octree pointers: 2-bit tag (0 node, 1 colour, 2 leaf, 3 null) above 30 bits
// of data (node index, RGB8 colour, leaf word index).  Nodes are 8 pointers,
// appended in JoinNode (post) order.  A leaf block in the word vector is
// [block size][macro count M][block count B][weight word count W]
// [M macro blocks: first block, weight start][B block headers: colours,
// voxel offset:14 | bits per weight:2 | weight offset:16][W weight words].
//
// A colour leaf covers the 8^(voxel_level - leaf_level) voxels under an octree
// node at leaf_level, in Morton order (bit 3k = x_k, 3k+1 = y_k, 3k+2 = z_k,
// finest first; the order in which the edit recursion visits children and
// leaf voxels, NodeCoord.hpp:18-43).  The chunk the reference's VBRChunkWriter
// produces depends only on the per-voxel sequence of (colours, bits per
// weight, weight): a block starts at every voxel whose (colours, bits per
// weight) differ from the previous voxel's and at every macro block start
// (every 2^14 voxels); the weight bits are the voxels' weights back to back.
// The colour rules of the editors (src/main.cpp:48-69,107-148) under the
// wrapper give every voxel of an edited leaf its colour:
//   walking from the colour leaf down through the old DAG, the first node that
//   the edit covers (kFill) or that is empty gives the edit's colour to its
//   whole subtree; the first node the edit does not touch keeps the old
//   colours of its subtree; at a voxel, the edit's colour if the voxel is in
//   the shape or was empty, else its old colour.
// Fill and paint editors follow the same colour rules (paint only keeps the
// geometry).
static constexpr Word kTagNode = 0, kTagColor = 1, kTagLeaf = 2, kTagNull = 3;
static constexpr Word kColorNull = kTagNull << 30;
static constexpr Word kMacroBits = 14; // VBRInfo::kVoxelBitsPerMacroBlock
static inline Word cptr(Word tag, Word data) { return (tag << 30) | data; }
static inline Word ctag(Word p) { return p >> 30; }
static inline Word cdata(Word p) { return p & 0x3FFFFFFFu; }

struct VColor { // VBRColor (VBRColor.hpp:18-43)
	Word colors = 0, weight = 0, bpw = 0, has = 0;
	bool operator==(const VColor &o) const {
		return colors == o.colors && weight == o.weight && bpw == o.bpw && has == o.has;
	}
};

// VBRColor::Get (VBRColor.hpp:31-36) with RGB8Color/R5G6B5Color::Get
// (Color.hpp:24,42-45) and glm::mix = x * (1 - a) + y * a, in float.
static inline void vcolor_rgb(const VColor &c, float rgb[3]) {
	if (c.bpw == 0) {
		for (int k = 0; k < 3; ++k)
			rgb[k] = float((c.colors >> (8 * k)) & 0xFFu) / 255.0f;
		return;
	}
	const Word lo = c.colors & 0xFFFFu, hi = c.colors >> 16;
	const float x[3] = {float(lo & 0x1Fu) / 31.0f, float((lo >> 5) & 0x3Fu) / 63.0f, float((lo >> 11) & 0x1Fu) / 31.0f};
	const float y[3] = {float(hi & 0x1Fu) / 31.0f, float((hi >> 5) & 0x3Fu) / 63.0f, float((hi >> 11) & 0x1Fu) / 31.0f};
	const float a = float(c.weight) / float((1u << c.bpw) - 1u);
	for (int k = 0; k < 3; ++k) {
		const float p = x[k] * (1.0f - a), q = y[k] * a;
		rgb[k] = p + q;
	}
}
// DAGColorPool::FillNode (src/DAGColorPool.hpp:167-169): RGB8Color{color.Get()}
static inline Word vcolor_rgb8(const VColor &c) {
	float rgb[3];
	vcolor_rgb(c, rgb);
	Word out = 0;
	for (int k = 0; k < 3; ++k)
		out |= Word(uint8_t(rgb[k] * 255.0f)) << (8 * k);
	return out;
}
// DAGColorPool::GetFill (src/DAGColorPool.hpp:147-149)
static inline VColor fill_of(Word p) { return ctag(p) == kTagColor ? VColor{cdata(p), 0, 0, 1} : VColor{}; }

struct ColorPool {
	Word leaf_level = 0;
	bool keep_history = false;
	std::vector<Word> nodes;  // 8 pointers per node
	std::vector<Word> leaves; // leaf blocks

	// DAGColorPool::GetChild (src/DAGColorPool.hpp:142-146)
	Word child(Word p, Word c) const {
		return ctag(p) == kTagNode ? nodes[size_t(cdata(p)) * 8 + c] : (ctag(p) == kTagColor ? p : kColorNull);
	}
	// DAGColorPool::SetNode (src/DAGColorPool.hpp:150-165)
	Word set_node(Word p, const Word ch[8]) {
		bool all_null = true, all_same_color = ctag(ch[0]) == kTagColor;
		for (int c = 0; c < 8; ++c) {
			all_null = all_null && ctag(ch[c]) == kTagNull;
			all_same_color = all_same_color && ch[c] == ch[0];
		}
		if (all_null)
			return kColorNull;
		if (all_same_color)
			return ch[0];
		if (ctag(p) == kTagNode && std::equal(ch, ch + 8, nodes.begin() + size_t(cdata(p)) * 8))
			return p;
		const Word idx = Word(nodes.size() / 8);
		nodes.insert(nodes.end(), ch, ch + 8);
		return cptr(kTagNode, idx);
	}
	// DAGColorPool::SetLeaf (src/DAGColorPool.hpp:176-207); chunk = [M, B, W, ...]
	Word set_leaf(Word p, const std::vector<Word> &chunk) {
		const size_t data_size = chunk.size() + 1;
		size_t append_size = (data_size & 1) ? data_size + 1 : data_size;
		if (!keep_history && ctag(p) == kTagLeaf) {
			const size_t idx = cdata(p), block_size = leaves[idx];
			if (data_size <= block_size) {
				std::copy(chunk.begin(), chunk.end(), leaves.begin() + idx + 1);
				return p;
			}
			append_size = std::max(block_size << 1, append_size);
		}
		const size_t idx = leaves.size();
		leaves.resize(idx + append_size, 0u);
		leaves[idx] = Word(append_size);
		std::copy(chunk.begin(), chunk.end(), leaves.begin() + idx + 1);
		return cptr(kTagLeaf, Word(idx));
	}
};

struct VStream { // per-voxel colours of one colour leaf, Morton order
	std::vector<Word> colors;
	std::vector<uint8_t> bpw, weight;
	explicit VStream(size_t n) : colors(n), bpw(n), weight(n) {}
	void set(size_t m, const VColor &c) {
		colors[m] = c.colors;
		bpw[m] = uint8_t(c.bpw);
		weight[m] = uint8_t(c.weight);
	}
	VColor get(size_t m) const { return VColor{colors[m], weight[m], bpw[m], 1}; }
};

// Voxel colours of the chunk of leaf pointer p (VBRChunkIterator, VBRColor.hpp:286-365),
// or the octree node's fill colour everywhere (VBRChunkWriter::Copy/Edit of an empty source).
static VStream decode_leaf(const ColorPool &cp, Word p, size_t n) {
	VStream s(n);
	if (ctag(p) != kTagLeaf) {
		const VColor f = fill_of(p);
		for (size_t m = 0; m < n; ++m)
			s.set(m, f);
		return s;
	}
	const Word *w = cp.leaves.data() + cdata(p);
	const Word M = w[1], B = w[2];
	const Word *macro = w + 4, *hdr = macro + 2 * M, *bits = hdr + 2 * B;
	for (Word k = 0; k < M; ++k) {
		const Word first = macro[2 * k], end = k + 1 < M ? macro[2 * k + 2] : B, wstart = macro[2 * k + 1];
		for (Word b = first; b < end; ++b) {
			const Word v0 = hdr[2 * b + 1] >> 18, bpw = (hdr[2 * b + 1] >> 16) & 3u, woff = hdr[2 * b + 1] & 0xFFFFu;
			Word v1 = b + 1 < end ? hdr[2 * (b + 1) + 1] >> 18 : (1u << kMacroBits);
			for (Word v = v0; v < v1; ++v) {
				const size_t m = (size_t(k) << kMacroBits) + v;
				if (m >= n)
					break;
				Word wt = 0;
				if (bpw) {
					const size_t bit = size_t(wstart) + woff + size_t(v - v0) * bpw;
					const uint64_t two = uint64_t(bits[bit >> 5]) | (((bit >> 5) + 1 < w[3]) ? uint64_t(bits[(bit >> 5) + 1]) << 32 : 0);
					wt = Word(two >> (bit & 31)) & ((1u << bpw) - 1u);
				}
				s.set(m, VColor{hdr[2 * b], wt, bpw, 1});
			}
		}
	}
	return s;
}

// VBRChunkWriter (VBRColor.hpp:367-488) output for a per-voxel colour sequence:
// [M, B, W, macro blocks, block headers, weight words].
static std::vector<Word> encode_leaf(const VStream &s) {
	const size_t n = s.colors.size();
	const size_t M = (n + (size_t(1) << kMacroBits) - 1) >> kMacroBits;
	std::vector<Word> macros, hdrs, wbits;
	uint64_t bit = 0, macro_wstart = 0;
	for (size_t m = 0; m < n; ++m) {
		const bool macro_start = (m & ((size_t(1) << kMacroBits) - 1)) == 0;
		if (macro_start) {
			macro_wstart = bit;
			macros.push_back(Word(hdrs.size() / 2));
			macros.push_back(Word(bit));
		}
		if (macro_start || s.colors[m] != s.colors[m - 1] || s.bpw[m] != s.bpw[m - 1]) {
			hdrs.push_back(s.colors[m]);
			hdrs.push_back(Word((m & ((size_t(1) << kMacroBits) - 1)) << 18) | (Word(s.bpw[m]) << 16) |
			               Word(bit - macro_wstart));
		}
		for (Word b = 0; b < s.bpw[m]; ++b, ++bit) {
			if ((bit & 31) == 0)
				wbits.push_back(0u);
			wbits.back() |= Word((s.weight[m] >> b) & 1u) << (bit & 31);
		}
	}
	std::vector<Word> out = {Word(M), Word(hdrs.size() / 2), Word(wbits.size())};
	out.insert(out.end(), macros.begin(), macros.end());
	out.insert(out.end(), hdrs.begin(), hdrs.end());
	out.insert(out.end(), wbits.begin(), wbits.end());
	return out;
}

// New colours of the voxels [m0, m0 + 8^(V - level)) of a colour leaf being
// edited: VBREditorWrapper::EditNode/EditVoxel below the leaf level
// (VBREditor.hpp:61-80,82-90) with the editors' colour rules.
static void vbr_region(const Pool &dag, const hd_edit_desc &g, const VColor &C, Word level, const Word pos[3],
                       Word dptr, Word leaf_level, size_t m0, const VStream &src, VStream &dst) {
	const Word V = dag.cfg.voxel_level(), L = dag.cfg.node_levels();
	const size_t count = size_t(1) << (3 * (V - level));
	if (level > leaf_level) {
		const EditType t = edit_node_type(g, V, level, pos);
		if (t == kFill || dptr == kNull) {
			for (size_t k = 0; k < count; ++k)
				dst.set(m0 + k, C);
			return;
		}
		if (t == kNotAffected) {
			for (size_t k = 0; k < count; ++k)
				dst.set(m0 + k, src.get(m0 + k));
			return;
		}
	}
	if (level == L - 1) {
		const Word *p = dag.read_node(dptr);
		for (Word i = 0; i < 64; ++i) {
			const Word vp[3] = {(pos[0] << 2) | ((i >> 2) & 2u) | (i & 1u), (pos[1] << 2) | ((i >> 3) & 2u) | ((i >> 1) & 1u),
			                    (pos[2] << 2) | ((i >> 4) & 2u) | ((i >> 2) & 1u)};
			const bool old = (p[i >> 5] >> (i & 31)) & 1u;
			dst.set(m0 + i, (voxel_in_shape(g, vp) || !old) ? C : src.get(m0 + i));
		}
		return;
	}
	const std::array<Word, 9> u = dag.unpack(dptr);
	for (Word c = 0; c < 8; ++c) {
		Word cp[3];
		Pool::child_pos(pos, c, cp);
		vbr_region(dag, g, C, level + 1, cp, u[1 + c], leaf_level, m0 + c * (count >> 3), src, dst);
	}
}

// ---- the same leaf rewrite in runs.  The reference's writer copies and fills
// whole runs (VBRChunkIterator / VBRChunkWriter::Copy, Edit, VBRColor.hpp:286-488);
// this form does too: the new voxel sequence is a list of segments, each
// either "the edit's colour" or "the old colours of these voxels", and only the
// DAG leaves the edit partly covers are decided voxel by voxel.  Its chunk is
// word for word encode_leaf's of the per-voxel form (a test compares the two).
static bool g_vbr_per_voxel = false; // the per-voxel form above (tests compare the two)

struct SrcBlock {      // voxels [m0, m1) of one block of the old chunk
	uint64_t m0, m1;
	Word colors, bpw;
	uint64_t bit0;     // weight of voxel m: bpw bits at bit0 + (m - m0) * bpw
};
struct SrcChunk {
	std::vector<SrcBlock> blocks;
	const Word *bits = nullptr;
	Word n_words = 0;
	Word weight(uint64_t bit, Word bpw) const { // as decode_leaf reads it
		const uint64_t two = uint64_t(bits[bit >> 5]) | (((bit >> 5) + 1 < n_words) ? uint64_t(bits[(bit >> 5) + 1]) << 32 : 0);
		return Word(two >> (bit & 31)) & ((1u << bpw) - 1u);
	}
};
static SrcChunk source_blocks(const ColorPool &cp, Word p, size_t n) {
	SrcChunk s;
	if (ctag(p) != kTagLeaf) {
		const VColor f = fill_of(p);
		s.blocks.push_back({0, n, f.colors, f.bpw, 0});
		return s;
	}
	const Word *w = cp.leaves.data() + cdata(p);
	const Word M = w[1], B = w[2];
	const Word *macro = w + 4, *hdr = macro + 2 * M;
	s.bits = hdr + 2 * B;
	s.n_words = w[3];
	for (Word k = 0; k < M; ++k) {
		const Word first = macro[2 * k], end = k + 1 < M ? macro[2 * k + 2] : B, wstart = macro[2 * k + 1];
		for (Word b = first; b < end; ++b) {
			const Word v0 = hdr[2 * b + 1] >> 18, v1 = b + 1 < end ? hdr[2 * (b + 1) + 1] >> 18 : (1u << kMacroBits);
			const uint64_t m0 = (uint64_t(k) << kMacroBits) + v0, m1 = std::min<uint64_t>(n, (uint64_t(k) << kMacroBits) + v1);
			if (m0 < m1)
				s.blocks.push_back({m0, m1, hdr[2 * b], (hdr[2 * b + 1] >> 16) & 3u,
				                    uint64_t(wstart) + (hdr[2 * b + 1] & 0xFFFFu)});
		}
	}
	return s;
}

struct Seg {
	bool copy; // old colours of voxels [m, m + len), else the edit's colour
	uint64_t m, len;
};
static inline void push_seg(std::vector<Seg> &segs, bool copy, uint64_t m, uint64_t len) {
	if (!segs.empty() && segs.back().copy == copy && segs.back().m + segs.back().len == m)
		segs.back().len += len;
	else
		segs.push_back({copy, m, len});
}
// vbr_region as segments
static void vbr_region_runs(const Pool &dag, const hd_edit_desc &g, Word level, const Word pos[3], Word dptr,
                            Word leaf_level, uint64_t m0, std::vector<Seg> &segs) {
	const Word V = dag.cfg.voxel_level(), L = dag.cfg.node_levels();
	const uint64_t count = uint64_t(1) << (3 * (V - level));
	if (level > leaf_level) {
		const EditType t = edit_node_type(g, V, level, pos);
		if (t == kFill || dptr == kNull) {
			push_seg(segs, false, m0, count);
			return;
		}
		if (t == kNotAffected) {
			push_seg(segs, true, m0, count);
			return;
		}
	}
	if (level == L - 1) {
		const Word *p = dag.read_node(dptr);
		for (Word i = 0; i < 64; ++i) {
			const Word vp[3] = {(pos[0] << 2) | ((i >> 2) & 2u) | (i & 1u), (pos[1] << 2) | ((i >> 3) & 2u) | ((i >> 1) & 1u),
			                    (pos[2] << 2) | ((i >> 4) & 2u) | ((i >> 2) & 1u)};
			const bool old = (p[i >> 5] >> (i & 31)) & 1u;
			push_seg(segs, !(voxel_in_shape(g, vp) || !old), m0 + i, 1);
		}
		return;
	}
	const std::array<Word, 9> u = dag.unpack(dptr);
	for (Word c = 0; c < 8; ++c) {
		Word cp[3];
		Pool::child_pos(pos, c, cp);
		vbr_region_runs(dag, g, level + 1, cp, u[1 + c], leaf_level, m0 + c * (count >> 3), segs);
	}
}

// encode_leaf fed by pieces of one colour instead of single voxels
struct RunEncoder {
	std::vector<Word> macros, hdrs, wbits;
	uint64_t bit = 0, macro_wstart = 0;
	Word pc = 0, pb = 0;
	void put_bits(Word v, Word nb) {
		for (Word b = 0; b < nb; ++b, ++bit) {
			if ((bit & 31) == 0)
				wbits.push_back(0u);
			wbits.back() |= ((v >> b) & 1u) << (bit & 31);
		}
	}
	// voxels [m, m + len) of colour (colors, bpw); weight(k) of voxel m + k
	template <typename WeightF> void piece(uint64_t m, uint64_t len, Word colors, Word bpw, WeightF &&weight) {
		const uint64_t macro_mask = (uint64_t(1) << kMacroBits) - 1;
		for (uint64_t k = 0; k < len;) {
			const uint64_t mm = m + k, in_macro = mm & macro_mask;
			const uint64_t chunk = std::min(len - k, (macro_mask + 1) - in_macro);
			if (in_macro == 0) {
				macro_wstart = bit;
				macros.push_back(Word(hdrs.size() / 2));
				macros.push_back(Word(bit));
			}
			if (in_macro == 0 || colors != pc || bpw != pb) {
				hdrs.push_back(colors);
				hdrs.push_back(Word(in_macro << 18) | (bpw << 16) | Word(bit - macro_wstart));
			}
			pc = colors;
			pb = bpw;
			if (bpw)
				for (uint64_t j = 0; j < chunk; ++j)
					put_bits(weight(k + j), bpw);
			k += chunk;
		}
	}
	std::vector<Word> chunk(size_t n) const {
		const size_t M = (n + (size_t(1) << kMacroBits) - 1) >> kMacroBits;
		std::vector<Word> out = {Word(M), Word(hdrs.size() / 2), Word(wbits.size())};
		out.insert(out.end(), macros.begin(), macros.end());
		out.insert(out.end(), hdrs.begin(), hdrs.end());
		out.insert(out.end(), wbits.begin(), wbits.end());
		return out;
	}
};

// The new chunk of a colour leaf being edited, in runs.
static std::vector<Word> vbr_leaf_runs(const ColorPool &cp, const Pool &dag, const hd_edit_desc &g, const VColor &C,
                                       Word level, const Word pos[3], Word optr, Word dptr) {
	const size_t n = size_t(1) << (3 * (dag.cfg.voxel_level() - level));
	const SrcChunk src = source_blocks(cp, optr, n);
	std::vector<Seg> segs;
	vbr_region_runs(dag, g, level, pos, dptr, cp.leaf_level, 0, segs);
	RunEncoder enc;
	size_t bi = 0;
	for (const Seg &sg : segs) {
		if (!sg.copy) {
			enc.piece(sg.m, sg.len, C.colors, C.bpw, [&](uint64_t) { return C.weight; });
			continue;
		}
		uint64_t m = sg.m;
		const uint64_t end = sg.m + sg.len;
		while (m < end) {
			while (bi < src.blocks.size() && src.blocks[bi].m1 <= m)
				++bi;
			if (bi == src.blocks.size() || src.blocks[bi].m0 > m) { // not covered by the old chunk: zeros
				const uint64_t e = bi == src.blocks.size() ? end : std::min(end, src.blocks[bi].m0);
				enc.piece(m, e - m, 0u, 0u, [](uint64_t) { return 0u; });
				m = e;
				continue;
			}
			const SrcBlock &b = src.blocks[bi];
			const uint64_t e = std::min(end, b.m1), base = b.bit0 + (m - b.m0) * b.bpw;
			enc.piece(m, e - m, b.colors, b.bpw, [&](uint64_t k) { return src.weight(base + k * b.bpw, b.bpw); });
			m = e;
		}
	}
	return enc.chunk(n);
}

// The colour octree part of one VBR edit at or above the colour leaf level:
// VBREditorWrapper::EditNode/JoinNode (VBREditor.hpp:40-80,92-107) with
// FillNode/ClearNode/SetNode/SetLeaf.  Returns the node's new pointer.
static Word vbr_walk(ColorPool &cp, const Pool &dag, const hd_edit_desc &g, const VColor &C, Word level,
                     const Word pos[3], Word optr, Word dptr) {
	const Word V = dag.cfg.voxel_level();
	const EditType t = edit_node_type(g, V, level, pos);
	if (t == kFill || dptr == kNull || fill_of(optr) == C)
		return cptr(kTagColor, vcolor_rgb8(C));
	if (t == kNotAffected)
		return optr;
	if (level == cp.leaf_level) {
		if (!g_vbr_per_voxel)
			return cp.set_leaf(optr, vbr_leaf_runs(cp, dag, g, C, level, pos, optr, dptr));
		const size_t n = size_t(1) << (3 * (V - level));
		const VStream src = decode_leaf(cp, optr, n);
		VStream dst(n);
		vbr_region(dag, g, C, level, pos, dptr, cp.leaf_level, 0, src, dst);
		return cp.set_leaf(optr, encode_leaf(dst));
	}
	const std::array<Word, 9> u = dag.unpack(dptr);
	Word ch[8];
	for (Word c = 0; c < 8; ++c) {
		Word cpos[3];
		Pool::child_pos(pos, c, cpos);
		ch[c] = vbr_walk(cp, dag, g, C, level + 1, cpos, cp.child(optr, c), u[1 + c]);
	}
	return cp.set_node(optr, ch);
}

// Colour of one voxel: Color_Fetch / Color_GetLeafColor (trace.frag:303-356).
static VColor color_fetch(const ColorPool &cp, Word root, Word voxel_level, const Word v[3]) {
	Word p = root;
	for (Word l = 0; l < cp.leaf_level && ctag(p) == kTagNode; ++l) {
		const Word s = voxel_level - 1u - l;
		p = cp.nodes[size_t(cdata(p)) * 8 + (((v[0] >> s) & 1u) | (((v[1] >> s) & 1u) << 1) | (((v[2] >> s) & 1u) << 2))];
	}
	if (ctag(p) != kTagLeaf)
		return ctag(p) == kTagColor ? fill_of(p) : VColor{};
	const Word bits = voxel_level - cp.leaf_level;
	Word vox = 0;
	for (Word b = 0; b < bits; ++b)
		vox |= (((v[0] >> b) & 1u) << (3 * b)) | (((v[1] >> b) & 1u) << (3 * b + 1)) | (((v[2] >> b) & 1u) << (3 * b + 2));
	const Word *w = cp.leaves.data() + cdata(p);
	const Word M = w[1];
	Word nb = w[2];
	const Word *macro = w + 4, *hdr = macro + 2 * M, *wb = hdr + 2 * nb;
	const Word mid = vox >> kMacroBits;
	if (mid >= M)
		return VColor{0, 0, 0, 1};
	const Word first = macro[2 * mid], wstart = macro[2 * mid + 1];
	Word cnt = mid + 1 < M ? macro[2 * mid + 2] - first : nb - first;
	const Word *b = hdr + 2 * first;
	vox &= (1u << kMacroBits) - 1u;
	if (cnt == 0)
		return VColor{0, 0, 0, 1};
	for (Word it = 0; it <= 14u && cnt != 0; ++it) { // first block whose voxel offset is > vox
		const Word step = cnt >> 1;
		if ((b[2 * step + 1] >> 18) <= vox) {
			cnt -= step + 1;
			b += 2 * (step + 1);
		} else
			cnt = step;
	}
	b -= 2;
	const Word bpw = (b[1] >> 16) & 3u;
	if (bpw == 0)
		return VColor{b[0], 0, 0, 1};
	const Word bit = wstart + (b[1] & 0xFFFFu) + (vox - (b[1] >> 18)) * bpw, off = bit & 31u;
	Word wt = wb[bit >> 5] >> off;
	if (off + bpw <= 32)
		wt &= (1u << bpw) - 1u;
	else
		wt |= (wb[(bit >> 5) + 1] & ((1u << (off + bpw - 32u)) - 1u)) << (32u - off);
	return VColor{b[0], wt, bpw, 1};
}

} // namespace orc

// ---------------------------------------------------------------- C ABI
using orc::Pool;
using orc::Word;

struct orc_pool {
	Pool pool;
	bool ok = true; // cleared when a bucket overflowed (reference: silent fallback)
	explicit orc_pool(orc::Config c) : pool(std::move(c)) {}
};

extern "C" {

orc_pool *orc_pool_create(uint32_t wbpp, uint32_t pbpb, uint32_t node_levels, const uint32_t *bucket_bits,
                          uint32_t hasher) {
	orc::Config c;
	c.wbpp = wbpp;
	c.pbpb = pbpb;
	c.hasher = hasher;
	c.bucket_bits.assign(bucket_bits, bucket_bits + node_levels);
	return new orc_pool(std::move(c));
}

void orc_pool_destroy(orc_pool *p) { delete p; }

int orc_pool_ok(const orc_pool *p) { return p->ok ? 1 : 0; }

void orc_make_filled(orc_pool *p, uint32_t *out) {
	p->pool.make_filled(&p->ok);
	if (out)
		for (size_t i = 0; i < p->pool.filled.size(); ++i)
			out[i] = p->pool.filled[i];
}

// Serial edits applied one after another (NodePoolBase::Edit per edit).
uint32_t orc_edit(orc_pool *p, uint32_t root, const hd_edit_desc *e, uint32_t n) {
	for (uint32_t i = 0; i < n; ++i)
		root = p->pool.edit(root, e[i], &p->ok);
	return root;
}

// Threaded edits (NodePoolThreadedEdit::ThreadedEdit per edit).
uint32_t orc_threaded_edit(orc_pool *p, uint32_t root, const hd_edit_desc *e, uint32_t n, uint32_t max_task_level,
                           int threads) {
	return p->pool.threaded_edits(root, e, n, max_task_level, threads, &p->ok);
}

int orc_max_threads(void) {
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

uint32_t orc_upsert(orc_pool *p, uint32_t level, const uint32_t *words, uint32_t len) {
	bool leaf = level == p->pool.cfg.node_levels() - 1;
	bool ok = true;
	Word r = p->pool.upsert<false>(leaf, level, words, len, orc::kNull, &ok);
	return ok ? r : orc::kNull;
}

uint32_t orc_bucket_words(const orc_pool *p, uint32_t bucket) { return p->pool.bucket_words[bucket]; }

uint64_t orc_total_buckets(const orc_pool *p) { return p->pool.cfg.total_buckets(); }
uint64_t orc_total_pages(const orc_pool *p) { return p->pool.cfg.total_pages(); }

// 1 if the virtual page exists, copies its words to out when out != NULL
int orc_read_page(const orc_pool *p, uint32_t page, uint32_t *out) {
	if (page >= p->pool.pages.size() || !p->pool.pages[page])
		return 0;
	if (out)
		std::memcpy(out, p->pool.pages[page].get(), size_t(p->pool.cfg.words_per_page()) * 4);
	return 1;
}

// Replace the pool contents (e.g. with a pool downloaded from the GPU).
void orc_pool_load(orc_pool *p, const uint32_t *bucket_words, const uint32_t *page_ids, uint32_t n_pages,
                   const uint32_t *page_words, const uint32_t *filled) {
	auto &pool = p->pool;
	uint64_t tb = pool.cfg.total_buckets();
	std::memcpy(pool.bucket_words.get(), bucket_words, tb * 4);
	for (auto &pg : pool.pages)
		pg.reset();
	Word wpp = pool.cfg.words_per_page();
	for (uint32_t i = 0; i < n_pages; ++i) {
		Word *dst = pool.page_for_write(page_ids[i]);
		std::memcpy(dst, page_words + size_t(i) * wpp, size_t(wpp) * 4);
	}
	if (filled)
		pool.filled.assign(filled, filled + pool.cfg.node_levels());
}

// Per-level canonical node counts and digests; returns 1 if the reachable DAG
// is fully reduced (no duplicate node content on a level) and well formed.
int orc_canonical(const orc_pool *p, uint32_t root, uint64_t *counts, uint64_t *digests) {
	orc::Canon c = orc::canonical(p->pool, root);
	if (c.bad_level >= 0)
		counts[0] = ~0ull - uint64_t(c.bad_level); // marks where the walk stopped
	for (size_t i = 0; i < c.counts.size(); ++i) {
		counts[i] = c.counts[i];
		digests[i] = c.digests[i];
	}
	return c.ok ? 1 : 0;
}

// The node-by-node canonicaliser (the cross-check of orc_canonical).
int orc_canonical_simple(const orc_pool *p, uint32_t root, uint64_t *counts, uint64_t *digests) {
	orc::Canon c = orc::canonical_simple(p->pool, root);
	if (c.bad_level >= 0)
		counts[0] = ~0ull - uint64_t(c.bad_level);
	for (size_t i = 0; i < c.counts.size(); ++i) {
		counts[i] = c.counts[i];
		digests[i] = c.digests[i];
	}
	return c.ok ? 1 : 0;
}

void orc_query(const orc_pool *p, uint32_t root, const uint32_t *xyz, uint32_t n, uint8_t *out) {
	for (uint32_t i = 0; i < n; ++i)
		out[i] = p->pool.query(root, xyz + 3 * size_t(i)) ? 1 : 0;
}

// Dense occupancy of the whole grid (small resolutions only): out[x + y*R + z*R*R].
void orc_dense(const orc_pool *p, uint32_t root, uint8_t *out) {
	Word R = 1u << p->pool.cfg.voxel_level();
	for (Word z = 0; z < R; ++z)
		for (Word y = 0; y < R; ++y)
			for (Word x = 0; x < R; ++x) {
				Word v[3] = {x, y, z};
				out[x + size_t(y) * R + size_t(z) * R * R] = p->pool.query(root, v) ? 1 : 0;
			}
}

void orc_trace(const orc_pool *p, uint32_t root, const float *o, const float *d, uint32_t n, hd_hit *out) {
	for (uint32_t i = 0; i < n; ++i)
		out[i] = orc::trace_ray(p->pool, root, o + 3 * size_t(i), d + 3 * size_t(i));
}

void orc_trace_threads(const orc_pool *p, uint32_t root, const float *o, const float *d, uint32_t n, hd_hit *out,
                       int threads) {
#pragma omp parallel for num_threads(threads) schedule(dynamic, 4096)
	for (int64_t i = 0; i < int64_t(n); ++i)
		out[i] = orc::trace_ray(p->pool, root, o + 3 * size_t(i), d + 3 * size_t(i));
}

void orc_trace_pinhole_lod(const orc_pool *p, uint32_t root, const hd_camera *cams, uint32_t n_cams, uint32_t w,
                           uint32_t h, float proj, float beam_proj, hd_hit *out, int threads) {
	orc::trace_pinhole_lod(p->pool, root, cams, n_cams, w, h, proj, beam_proj, out, threads);
}

// ThreadedGC restated: threads 0 = all; the result does not depend on it.
void orc_gc(orc_pool *p, uint32_t *roots, uint32_t n_roots, int threads) {
	p->pool.gc(roots, n_roots, &p->ok, threads);
}
// The one-thread form kept as the cross-check of orc_gc (same words).
void orc_gc_serial(orc_pool *p, uint32_t *roots, uint32_t n_roots) { p->pool.gc_serial(roots, n_roots, &p->ok); }

// ---- VBR colour (test infrastructure)
struct orc_color_pool {
	orc::ColorPool cp;
};
orc_color_pool *orc_color_pool_create(uint32_t leaf_level, int keep_history) {
	auto *c = new orc_color_pool;
	c->cp.leaf_level = leaf_level;
	c->cp.keep_history = keep_history != 0;
	return c;
}
void orc_color_pool_destroy(orc_color_pool *c) { delete c; }
uint64_t orc_color_nodes(const orc_color_pool *c, uint32_t *out) {
	if (out)
		std::copy(c->cp.nodes.begin(), c->cp.nodes.end(), out);
	return c->cp.nodes.size() / 8;
}
uint64_t orc_color_leaves(const orc_color_pool *c, uint32_t *out) {
	if (out)
		std::copy(c->cp.leaves.begin(), c->cp.leaves.end(), out);
	return c->cp.leaves.size();
}
void orc_color_pool_load(orc_color_pool *c, const uint32_t *nodes, uint64_t n_nodes, const uint32_t *leaves,
                         uint64_t n_words) {
	c->cp.nodes.assign(nodes, nodes + 8 * n_nodes);
	c->cp.leaves.assign(leaves, leaves + n_words);
}
// One VBR edit (kind 1 fill, 2 paint; colour = colors/weight/bpw): the colour
// octree from the old DAG root, then the geometry (fill only).
void orc_vbr_edit(orc_pool *p, orc_color_pool *c, uint32_t root, uint32_t color_root, const hd_edit_desc *e,
                  uint32_t kind, uint32_t colors, uint32_t weight, uint32_t bpw, uint32_t *out_root,
                  uint32_t *out_color_root) {
	hd_edit_desc g = *e;
	g.op = HD_OP_FILL;
	p->pool.make_filled(&p->ok);
	const orc::VColor C{colors, weight, bpw, 1};
	const orc::Word zero[3] = {0, 0, 0};
	*out_color_root = orc::vbr_walk(c->cp, p->pool, g, C, 0, zero, color_root, root);
	*out_root = kind == 2 ? root : p->pool.edit(root, g, &p->ok);
}
// Colour of voxels (x,y,z triples): has_value, colors, weight, bpw, rgb[3] (float bits).
void orc_color_fetch(const orc_pool *p, const orc_color_pool *c, uint32_t color_root, const uint32_t *xyz, uint32_t n,
                     uint32_t *out) {
	for (uint32_t i = 0; i < n; ++i) {
		const orc::VColor v = orc::color_fetch(c->cp, color_root, p->pool.cfg.voxel_level(), xyz + 3 * i);
		float rgb[3];
		orc::vcolor_rgb(v, rgb);
		uint32_t *o = out + 7 * size_t(i);
		o[0] = v.has;
		o[1] = v.colors;
		o[2] = v.weight;
		o[3] = v.bpw;
		std::memcpy(o + 4, rgb, 12);
	}
}

// 1: colour leaves rewritten voxel by voxel; 0 (default): in runs.  The two
// give the same words; tests compare them.
void orc_vbr_set_per_voxel(int on) { orc::g_vbr_per_voxel = on != 0; }

uint32_t orc_hash_inner(const uint32_t *w, uint32_t n) { return orc::murmur_words(w, n); }
uint32_t orc_hash_leaf(uint32_t w0, uint32_t w1) { return orc::murmur_leaf(w0, w1); }

// Voxel-edits of an edit list: the number of grid voxels of [0,res)^3 inside
// each edit's shape (VoxelInRange of src/main.cpp:55-57,121-126), summed.  A
// sphere is counted row by row: for every (y, z) row the x extent is
// cx +- isqrt(r2 - dy^2 - dz^2), clipped to the grid; spheres that lie inside
// the grid depend only on r2 and are counted once per r2.
// floor(sqrt(v)): a double estimate corrected in integers (no long double:
// on aarch64 that is a software quad-precision type, about 30x slower here).
static uint64_t isqrt_u64(uint64_t v) {
	uint64_t r = (uint64_t)std::sqrt((double)v);
	if (r > 0xFFFFFFFFull)
		r = 0xFFFFFFFFull;
	while (r * r > v)
		--r;
	while (r < 0xFFFFFFFFull && (r + 1) * (r + 1) <= v)
		++r;
	return r;
}
static uint64_t sphere_voxels(int64_t cx, int64_t cy, int64_t cz, uint64_t r2, int64_t res) {
	const int64_t r = (int64_t)isqrt_u64(r2);
	uint64_t total = 0;
	for (int64_t z = std::max<int64_t>(0, cz - r); z <= std::min<int64_t>(res - 1, cz + r); ++z) {
		const uint64_t dz2 = uint64_t((z - cz) * (z - cz));
		for (int64_t y = std::max<int64_t>(0, cy - r); y <= std::min<int64_t>(res - 1, cy + r); ++y) {
			const uint64_t d2 = dz2 + uint64_t((y - cy) * (y - cy));
			if (d2 > r2)
				continue;
			const int64_t w = (int64_t)isqrt_u64(r2 - d2);
			const int64_t lo = std::max<int64_t>(0, cx - w), hi = std::min<int64_t>(res - 1, cx + w);
			if (hi >= lo)
				total += uint64_t(hi - lo + 1);
		}
	}
	return total;
}
uint64_t orc_count_voxel_edits(const hd_edit_desc *e, uint32_t n, uint32_t res) {
	std::unordered_map<uint64_t, uint64_t> inside; // r2 -> voxels of a sphere inside the grid
	uint64_t total = 0;
	for (uint32_t i = 0; i < n; ++i) {
		if (e[i].shape == HD_SHAPE_AABB) {
			uint64_t v = 1;
			for (int a = 0; a < 3; ++a) {
				const uint64_t lo = std::min<uint64_t>(e[i].p0[a], res), hi = std::min<uint64_t>(e[i].p1[a], res);
				v *= hi > lo ? hi - lo : 0;
			}
			total += v;
			continue;
		}
		const int64_t r = (int64_t)isqrt_u64(e[i].r2);
		bool in = true;
		for (int a = 0; a < 3; ++a)
			in = in && int64_t(e[i].p0[a]) - r >= 0 && int64_t(e[i].p0[a]) + r < int64_t(res);
		if (in) {
			auto it = inside.find(e[i].r2);
			if (it == inside.end())
				it = inside.emplace(e[i].r2, sphere_voxels(r, r, r, e[i].r2, 2 * r + 1)).first;
			total += it->second;
		} else
			total += sphere_voxels(e[i].p0[0], e[i].p0[1], e[i].p0[2], e[i].r2, res);
	}
	return total;
}

} // extern "C"
