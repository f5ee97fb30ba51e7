/* hashdag_host_mirror.hpp -- host copy of a HashDAG pool in the reference's
 * storage layout, with the reference's storage hooks.
 *
 * The reference's pool algorithms (NodePoolBase::Edit, NodePoolThreadedEdit,
 * NodePoolThreadedGC, NodePoolTraversal) reach storage only through the hooks
 * of its NodePool / ThreadedNodePool / GCNodePool concepts
 * (include/hashdag/NodePool.hpp:22-38), implemented by the application's
 * DAGNodePool (src/DAGNodePool.hpp:56-74): bucket word counts, pages of
 * 2^word_bits_per_page words allocated on first write, a mutex per bucket
 * group, page release, and the written range of every page and the freed
 * pages that its Flush sends to the renderer (src/DAGNodePool.hpp:62-69,
 * src/DAGNodePool.cpp:56-85).  HostPoolMirror holds exactly that state, with
 * those hooks and their signatures, so a class deriving from it and from the
 * reference's CRTP bases (plus `using WordSpanHasher = ...`) runs the
 * reference's algorithms on it.  GpuNodePool (hashdag_gpu_pool.hpp) fills it
 * from a device pool, incrementally, and writes it back.
 *
 * Save / Load write and read a pool dump (a checkpoint file):
 *   "HDMP", version 1, the hd_config (as in hashdag_gpu.h), total buckets,
 *   bucket word counts, number of pages, then per page its id and words;
 *   all little-endian uint32.
 *
 * Header-only C++20; needs neither CUDA nor the GB300 library.
 */
#pragma once

#include "hashdag_gpu.h"

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <span>
#include <vector>

namespace hashdag_gb300 {

/* Derived sizes of a pool configuration (Config::GetTotalBuckets / GetTotalPages /
 * GetWordsPerPage, include/hashdag/Config.hpp:24,39-45). */
inline uint32_t config_total_buckets(const hd_config &c) {
	uint32_t n = 0;
	for (uint32_t l = 0; l < c.node_levels && l < HD_MAX_LEVELS; ++l)
		n += 1u << c.bucket_bits_each_level[l];
	return n;
}
inline uint32_t config_total_pages(const hd_config &c) { return config_total_buckets(c) << c.page_bits_per_bucket; }
inline uint32_t config_words_per_page(const hd_config &c) { return 1u << c.word_bits_per_page; }
/* The configuration with the bucket bits past node_levels zeroed (the form a dump stores). */
inline hd_config config_normalized(const hd_config &c) {
	hd_config n = c;
	for (uint32_t l = c.node_levels; l < HD_MAX_LEVELS; ++l)
		n.bucket_bits_each_level[l] = 0;
	return n;
}

/* Words [begin, end) of one page (Range<uint32_t> of the application). */
struct PageRange {
	uint32_t begin = 0, end = 0;
	bool empty() const { return begin >= end; }
	void unite(uint32_t b, uint32_t e) {
		if (b >= e)
			return;
		if (empty()) {
			begin = b, end = e;
		} else {
			begin = std::min(begin, b);
			end = std::max(end, e);
		}
	}
	bool operator==(const PageRange &o) const { return begin == o.begin && end == o.end; }
};

/* One page that appending passes wrote to, and the words they wrote there. */
struct AppendedPage {
	uint32_t page_id;
	PageRange words;
};

class HostPoolMirror {
public:
	explicit HostPoolMirror(const hd_config &config)
	    : mir_config(config), mir_bucket_words(config_total_buckets(config), 0u), mir_pages(config_total_pages(config)),
	      mir_written(config_total_pages(config)), mir_freed(config_total_pages(config), 0u) {}
	HostPoolMirror(const HostPoolMirror &) = delete;
	HostPoolMirror &operator=(const HostPoolMirror &) = delete;

	/* ---- the reference's storage hooks (signatures of src/DAGNodePool.hpp:56-74) */
	/* NodePool: words in use per bucket (the append cursor of upsert_node). */
	uint32_t &GetBucketRefWords(uint32_t bucket_id) { return mir_bucket_words[bucket_id]; }
	/* NodePool: the words of a page; null for a page never written. */
	const uint32_t *ReadPage(uint32_t page_id) const { return mir_pages[page_id].get(); }
	/* NodePool: zero a page range (append_node's padding; the page is created if
	 * needed).  The range counts as written. */
	void ZeroPage(uint32_t page_id, uint32_t page_offset, uint32_t zero_words) {
		uint32_t *p = page_for_write(page_id);
		std::fill(p + page_offset, p + page_offset + zero_words, 0u);
		mir_written[page_id].unite(page_offset, page_offset + zero_words);
	}
	/* NodePool: write words at an offset of a page (created zeroed on first write). */
	void WritePage(uint32_t page_id, uint32_t page_offset, std::span<const uint32_t> word_span) {
		std::copy(word_span.begin(), word_span.end(), page_for_write(page_id) + page_offset);
		mir_written[page_id].unite(page_offset, page_offset + (uint32_t)word_span.size());
	}
	/* ThreadedNodePool: the lock of a bucket (one of 1024, by bucket id). */
	std::mutex &GetBucketRefMutex(uint32_t bucket_id) { return mir_mutexes[bucket_id % mir_mutexes.size()]; }
	/* GCNodePool: release a page. */
	void FreePage(uint32_t page_id) {
		mir_pages[page_id].reset();
		mir_written[page_id] = PageRange{};
		mir_freed[page_id] = 1;
	}

	/* ---- mirror bookkeeping */
	const hd_config &MirrorConfig() const { return mir_config; }
	uint32_t TotalBuckets() const { return (uint32_t)mir_bucket_words.size(); }
	uint32_t TotalPages() const { return (uint32_t)mir_pages.size(); }
	uint32_t WordsPerPage() const { return config_words_per_page(mir_config); }
	bool HasPage(uint32_t page_id) const { return (bool)mir_pages[page_id]; }
	const std::vector<uint32_t> &BucketWords() const { return mir_bucket_words; }
	/* What changed since the last ClearDirty, as the application's Flush sends
	 * it (src/DAGNodePool.cpp:56-85): the written word range of a page, and
	 * whether the page was freed (and not written again). */
	PageRange WrittenRange(uint32_t page_id) const { return mir_written[page_id]; }
	bool IsFreed(uint32_t page_id) const { return mir_freed[page_id] != 0; }
	bool IsDirty(uint32_t page_id) const { return !mir_written[page_id].empty() || mir_freed[page_id]; }
	/* Records words of a page as written without changing them. */
	void MarkWritten(uint32_t page_id, PageRange words) { mir_written[page_id].unite(words.begin, words.end); }
	void ClearDirty() {
		std::fill(mir_written.begin(), mir_written.end(), PageRange{});
		std::fill(mir_freed.begin(), mir_freed.end(), 0u);
	}
	/* Pages that hold data, in ascending id order. */
	std::vector<uint32_t> PageIds() const {
		std::vector<uint32_t> ids;
		for (uint32_t i = 0; i < TotalPages(); ++i)
			if (mir_pages[i])
				ids.push_back(i);
		return ids;
	}
	/* Drops every page and bucket count (an empty pool, nothing dirty). */
	void Clear() {
		std::fill(mir_bucket_words.begin(), mir_bucket_words.end(), 0u);
		for (auto &p : mir_pages)
			p.reset();
		ClearDirty();
	}
	/* Installs one page's words as they are (the device copy), not marked dirty. */
	void SetPage(uint32_t page_id, const uint32_t *words) {
		uint32_t *p = page_for_write(page_id);
		std::copy(words, words + WordsPerPage(), p);
	}

	/* Pages an append-only pool wrote to when its bucket word counts went from
	 * the mirror's to new_counts: for every bucket whose count grew, the pages
	 * covering words [old, new) of the bucket with the words inside each page.
	 * False (and nothing appended to out) if any count went down: the pool was
	 * rewritten, not appended to. */
	bool AppendedPages(const std::vector<uint32_t> &new_counts, std::vector<AppendedPage> *out) const {
		if (new_counts.size() != mir_bucket_words.size())
			return false;
		for (uint32_t b = 0; b < TotalBuckets(); ++b)
			if (new_counts[b] < mir_bucket_words[b])
				return false;
		const uint32_t wbpp = mir_config.word_bits_per_page, wpp = WordsPerPage();
		for (uint32_t b = 0; b < TotalBuckets(); ++b) {
			const uint32_t lo = mir_bucket_words[b], hi = new_counts[b];
			if (hi <= lo)
				continue;
			const uint32_t p0 = lo >> wbpp, p1 = (hi - 1u) >> wbpp;
			for (uint32_t p = p0; p <= p1; ++p) {
				AppendedPage a;
				a.page_id = (b << mir_config.page_bits_per_bucket) | p;
				a.words.begin = p == p0 ? lo & (wpp - 1u) : 0u;
				a.words.end = p == p1 ? ((hi - 1u) & (wpp - 1u)) + 1u : wpp;
				out->push_back(a);
			}
		}
		return true;
	}

	/* ---- pool dumps */
	bool Save(const char *path) const {
		std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path, "wb"), &std::fclose);
		if (!f)
			return false;
		const std::vector<uint32_t> ids = PageIds();
		const hd_config c = config_normalized(mir_config);
		bool ok = std::fwrite("HDMP", 1, 4, f.get()) == 4 && put(f.get(), kDumpVersion) &&
		          std::fwrite(&c, sizeof(hd_config), 1, f.get()) == 1 && put(f.get(), TotalBuckets()) &&
		          std::fwrite(mir_bucket_words.data(), 4, TotalBuckets(), f.get()) == TotalBuckets() &&
		          put(f.get(), (uint32_t)ids.size());
		for (size_t k = 0; ok && k < ids.size(); ++k)
			ok = put(f.get(), ids[k]) && std::fwrite(ReadPage(ids[k]), 4, WordsPerPage(), f.get()) == WordsPerPage();
		return ok;
	}
	/* Reads a dump of a pool with this mirror's configuration into the mirror
	 * (every page it holds counts as written).  False, with the mirror
	 * cleared, on a malformed file or another configuration. */
	bool Load(const char *path) {
		Clear();
		std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path, "rb"), &std::fclose);
		if (!f)
			return false;
		char magic[4];
		hd_config c;
		const hd_config mine = config_normalized(mir_config);
		uint32_t version = 0, nb = 0, np = 0;
		if (std::fread(magic, 1, 4, f.get()) != 4 || std::memcmp(magic, "HDMP", 4) != 0 || !get(f.get(), &version) ||
		    version != kDumpVersion || std::fread(&c, sizeof(hd_config), 1, f.get()) != 1 ||
		    std::memcmp(&c, &mine, sizeof(hd_config)) != 0 || !get(f.get(), &nb) || nb != TotalBuckets() ||
		    std::fread(mir_bucket_words.data(), 4, nb, f.get()) != nb || !get(f.get(), &np) || np > TotalPages()) {
			Clear();
			return false;
		}
		std::vector<uint32_t> words(WordsPerPage());
		for (uint32_t k = 0; k < np; ++k) {
			uint32_t id = 0;
			if (!get(f.get(), &id) || id >= TotalPages() || HasPage(id) ||
			    std::fread(words.data(), 4, WordsPerPage(), f.get()) != WordsPerPage()) {
				Clear();
				return false;
			}
			WritePage(id, 0, std::span<const uint32_t>(words));
		}
		return true;
	}

private:
	static constexpr uint32_t kDumpVersion = 1;
	static bool put(FILE *f, uint32_t v) { return std::fwrite(&v, 4, 1, f) == 1; }
	static bool get(FILE *f, uint32_t *v) { return std::fread(v, 4, 1, f) == 1; }

	uint32_t *page_for_write(uint32_t page_id) {
		if (!mir_pages[page_id])
			mir_pages[page_id] = std::make_unique<uint32_t[]>(WordsPerPage()); // zeroed
		mir_freed[page_id] = 0;
		return mir_pages[page_id].get();
	}

	hd_config mir_config;
	std::vector<uint32_t> mir_bucket_words;
	std::vector<std::unique_ptr<uint32_t[]>> mir_pages;
	std::vector<PageRange> mir_written;
	std::vector<uint8_t> mir_freed;
	std::array<std::mutex, 1024> mir_mutexes{};
};

} // namespace hashdag_gb300
