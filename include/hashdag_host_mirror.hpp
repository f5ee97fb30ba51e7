/* hashdag_host_mirror.hpp -- host copy of a HashDAG pool in the reference's
 * storage layout, with the reference's storage hooks.
 *
 * The reference's pool algorithms (NodePoolBase::Edit, NodePoolThreadedEdit,
 * NodePoolThreadedGC, NodePoolTraversal) reach storage only through the hooks
 * of its NodePool / ThreadedNodePool / GCNodePool concepts
 * (include/hashdag/NodePool.hpp:22-38), implemented by the application's
 * DAGNodePool (src/DAGNodePool.hpp:56-74): bucket word counts, pages of
 * 2^word_bits_per_page words allocated on first write, a mutex per bucket
 * group, page release.  HostPoolMirror holds exactly that state, with those
 * hooks and their signatures, so a class deriving from it and from the
 * reference's CRTP bases (plus `using WordSpanHasher = ...`) runs the
 * reference's algorithms on it.  GpuNodePool (hashdag_gpu_pool.hpp) fills it
 * from a device pool and writes it back.
 *
 * Header-only C++20; needs neither CUDA nor the GB300 library.
 */
#pragma once

#include "hashdag_gpu.h"

#include <algorithm>
#include <array>
#include <cstdint>
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

class HostPoolMirror {
public:
	explicit HostPoolMirror(const hd_config &config)
	    : mir_config(config), mir_bucket_words(config_total_buckets(config), 0u), mir_pages(config_total_pages(config)),
	      mir_dirty(config_total_pages(config), 0u) {}
	HostPoolMirror(const HostPoolMirror &) = delete;
	HostPoolMirror &operator=(const HostPoolMirror &) = delete;

	/* ---- the reference's storage hooks (signatures of src/DAGNodePool.hpp:56-74) */
	/* NodePool: words in use per bucket (the append cursor of upsert_node). */
	uint32_t &GetBucketRefWords(uint32_t bucket_id) { return mir_bucket_words[bucket_id]; }
	/* NodePool: the words of a page; null for a page never written. */
	const uint32_t *ReadPage(uint32_t page_id) const { return mir_pages[page_id].get(); }
	/* NodePool: zero a page range (append_node's padding; the page is created if needed). */
	void ZeroPage(uint32_t page_id, uint32_t page_offset, uint32_t zero_words) {
		uint32_t *p = page_for_write(page_id);
		std::fill(p + page_offset, p + page_offset + zero_words, 0u);
	}
	/* NodePool: write words at an offset of a page (created zeroed on first write). */
	void WritePage(uint32_t page_id, uint32_t page_offset, std::span<const uint32_t> word_span) {
		std::copy(word_span.begin(), word_span.end(), page_for_write(page_id) + page_offset);
	}
	/* ThreadedNodePool: the lock of a bucket (one of 1024, by bucket id). */
	std::mutex &GetBucketRefMutex(uint32_t bucket_id) { return mir_mutexes[bucket_id % mir_mutexes.size()]; }
	/* GCNodePool: release a page. */
	void FreePage(uint32_t page_id) {
		mir_pages[page_id].reset();
		mir_dirty[page_id] = 1;
	}

	/* ---- mirror bookkeeping */
	const hd_config &MirrorConfig() const { return mir_config; }
	uint32_t TotalBuckets() const { return (uint32_t)mir_bucket_words.size(); }
	uint32_t TotalPages() const { return (uint32_t)mir_pages.size(); }
	uint32_t WordsPerPage() const { return config_words_per_page(mir_config); }
	bool HasPage(uint32_t page_id) const { return (bool)mir_pages[page_id]; }
	const std::vector<uint32_t> &BucketWords() const { return mir_bucket_words; }
	/* Pages written, zeroed or freed since the last ClearDirty: what the
	 * application's Flush would send to the device (src/DAGNodePool.cpp:56-85). */
	bool IsDirty(uint32_t page_id) const { return mir_dirty[page_id] != 0; }
	void ClearDirty() { std::fill(mir_dirty.begin(), mir_dirty.end(), 0u); }
	/* Pages that hold data, in ascending id order. */
	std::vector<uint32_t> PageIds() const {
		std::vector<uint32_t> ids;
		for (uint32_t i = 0; i < TotalPages(); ++i)
			if (mir_pages[i])
				ids.push_back(i);
		return ids;
	}
	/* Drops every page and bucket count (an empty pool). */
	void Clear() {
		std::fill(mir_bucket_words.begin(), mir_bucket_words.end(), 0u);
		for (auto &p : mir_pages)
			p.reset();
		ClearDirty();
	}
	/* Installs one page's words as they are (the device copy), not marked dirty. */
	void SetPage(uint32_t page_id, const uint32_t *words) {
		std::copy(words, words + WordsPerPage(), page_for_write(page_id));
		mir_dirty[page_id] = 0;
	}

private:
	uint32_t *page_for_write(uint32_t page_id) {
		if (!mir_pages[page_id])
			mir_pages[page_id] = std::make_unique<uint32_t[]>(WordsPerPage()); // zeroed
		mir_dirty[page_id] = 1;
		return mir_pages[page_id].get();
	}

	hd_config mir_config;
	std::vector<uint32_t> mir_bucket_words;
	std::vector<std::unique_ptr<uint32_t[]>> mir_pages;
	std::vector<uint8_t> mir_dirty;
	std::array<std::mutex, 1024> mir_mutexes{};
};

} // namespace hashdag_gb300
