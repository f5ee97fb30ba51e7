/* hashdag_gpu_pool.hpp -- C++ host side of a device HashDAG pool.
 *
 * GpuNodePool stands where the application's DAGNodePool stands
 * (src/DAGNodePool.hpp:31-105): it owns the pool (on the GB300, through the C
 * ABI of hashdag_gpu.h), takes edits root in / root out, keeps the root the
 * renderer reads, and holds a host mirror of the pool's words in the
 * reference's storage layout (HostPoolMirror).  GpuNodePool forwards the
 * mirror's storage hooks, so it satisfies the reference's NodePool,
 * ThreadedNodePool and GCNodePool concepts (include/hashdag/NodePool.hpp:22-38)
 * for code that reads or edits the host copy with the reference's own
 * algorithms.
 *
 *   auto pool = hashdag_gb300::GpuNodePool::Create(config);   // nullptr on failure
 *   uint32_t root = HD_NULL_PTR;
 *   pool->Edit(root, edits, &root);                          // one batched pass
 *   root = pool->ThreadedEdit(&busy_pool, root, SphereEditor<EditMode::kDig>{c, r2}, 10); // the app's call
 *   pool->Publish();                                         // device -> mirror, what changed
 *   ... flush pool->Mirror()'s written ranges and freed pages, ClearDirty ...
 *   ... or read / edit the mirror (ReadPage, GetBucketRefWords, ...) ...
 *   pool->Upload();                                          // mirror -> device
 *   pool->Mirror().Save("pool.hdmp");                        // a checkpoint file
 *
 * Header-only C++20 over libhashdag_gb300.so.  Every call returns the
 * library's hd_status; nothing falls back to the CPU.
 */
#pragma once

#include "hashdag_gpu.h"
#include "hashdag_host_mirror.hpp"

#include <algorithm>
#include <concepts>
#include <cstdint>
#include <memory>
#include <type_traits>
#include <mutex>
#include <span>
#include <vector>

namespace hashdag_gb300 {

/* ---- editors ---------------------------------------------------------------
 * The reference passes editors as compile-time objects (the Editor and
 * StatelessEditor concepts, include/hashdag/Editor.hpp:36-55) whose EditNode /
 * EditVoxel run inside its CPU recursion.  The device runs the shapes of the
 * application's editors (src/main.cpp:32-150) instead, so an editor object is
 * lowered to an hd_edit_desc at the boundary:
 *   - a sphere: members `center` (.x .y .z) and `r2` -- SphereEditor<Mode> of
 *     src/main.cpp:65-150, Mode from the application's EditMode (kFill = 0,
 *     kDig = 1, kPaint = 2; paint changes colours only, so it is accepted by
 *     the colour path alone);
 *   - a box: members `aabb_min` and `aabb_max` (.x .y .z) -- AABBEditor of
 *     src/main.cpp:32-63 (a fill); a class template with one mode argument and
 *     these members (e.g. a box editor with kDig) digs or paints by its mode;
 *   - any other type E: specialise EditorLowering<E> with
 *     `static hd_edit_desc Lower(const E &)` (and, for colour edits,
 *     `static hd_vbr_edit_desc LowerColor(const E &)`).
 * Anything else does not compile: there is no CPU path that could run an
 * arbitrary EditNode. */
template <class E> struct EditorLowering {};

namespace detail {
template <class V> concept Vec3 = requires(const V v) {
	{ v.x } -> std::convertible_to<uint32_t>;
	{ v.y } -> std::convertible_to<uint32_t>;
	{ v.z } -> std::convertible_to<uint32_t>;
};
template <class E> concept SphereShape = requires(const E e) {
	requires Vec3<decltype(e.center)>;
	{ e.r2 } -> std::convertible_to<uint64_t>;
};
template <class E> concept BoxShape = requires(const E e) {
	requires Vec3<decltype(e.aabb_min)>;
	requires Vec3<decltype(e.aabb_max)>;
};
// The mode argument of an editor class template (SphereEditor<EditMode::kDig>):
// its value as an integer in the application's EditMode order; -1 without one.
template <class E> struct ModeOf : std::integral_constant<int, -1> {};
template <template <auto> class T, auto M> struct ModeOf<T<M>> : std::integral_constant<int, static_cast<int>(M)> {};
// VBRColor (include/hashdag/VBRColor.hpp:18-43) through its accessors.
template <class C> concept VbrColorLike = requires(const C c) {
	{ c.GetColors() } -> std::convertible_to<uint32_t>;
	{ c.GetWeight() } -> std::convertible_to<uint32_t>;
	{ c.GetBitsPerWeight() } -> std::convertible_to<uint32_t>;
};
template <class E> concept ColorMember = requires(const E e) { requires VbrColorLike<decltype(e.color)>; };
template <class> inline constexpr bool kAlwaysFalse = false;
} // namespace detail

template <class E> concept CustomEditor = requires(const E e) {
	{ EditorLowering<E>::Lower(e) } -> std::same_as<hd_edit_desc>;
};
/* Editor types the device can apply to the geometry. */
template <class E> concept DeviceEditor =
    CustomEditor<E> || ((detail::SphereShape<E> || detail::BoxShape<E>) && detail::ModeOf<E>::value != 2);
/* Editor types the device can apply as colour edits (VBREditorWrapper,
 * include/hashdag/VBREditor.hpp:26-107): the shapes above with a `color`. */
template <class E> concept DeviceColorEditor =
    requires(const E e) {
	    { EditorLowering<E>::LowerColor(e) } -> std::same_as<hd_vbr_edit_desc>;
    } || ((detail::SphereShape<E> || detail::BoxShape<E>) && detail::ColorMember<E>);

namespace detail {
template <class E> hd_edit_desc lower_shape(const E &e, uint32_t op) {
	hd_edit_desc d{};
	d.op = op;
	if constexpr (SphereShape<E>) {
		d.shape = HD_SHAPE_SPHERE;
		d.p0[0] = (uint32_t)e.center.x;
		d.p0[1] = (uint32_t)e.center.y;
		d.p0[2] = (uint32_t)e.center.z;
		d.r2 = (uint64_t)e.r2;
	} else {
		d.shape = HD_SHAPE_AABB;
		d.p0[0] = (uint32_t)e.aabb_min.x;
		d.p0[1] = (uint32_t)e.aabb_min.y;
		d.p0[2] = (uint32_t)e.aabb_min.z;
		d.p1[0] = (uint32_t)e.aabb_max.x;
		d.p1[1] = (uint32_t)e.aabb_max.y;
		d.p1[2] = (uint32_t)e.aabb_max.z;
	}
	return d;
}
} // namespace detail

/* One editor object as the descriptor the device applies (geometry). */
template <class E> hd_edit_desc LowerEditor(const E &e) {
	if constexpr (CustomEditor<E>) {
		return EditorLowering<E>::Lower(e);
	} else if constexpr (DeviceEditor<E>) {
		constexpr int mode = detail::ModeOf<E>::value;
		static_assert(mode == -1 || mode == 0 || mode == 1, "unknown editor mode (EditMode: kFill, kDig, kPaint)");
		return detail::lower_shape(e, mode == 1 ? HD_OP_DIG : HD_OP_FILL);
	} else {
		static_assert(detail::kAlwaysFalse<E>, "not an editor the device can apply: give it center/r2 or "
		                                       "aabb_min/aabb_max, or specialise hashdag_gb300::EditorLowering");
		return {};
	}
}
/* One colour editor object as a colour edit (its shape, its mode -- fill, or
 * paint for EditMode::kPaint -- and its VBRColor). */
template <class E> hd_vbr_edit_desc LowerColorEditor(const E &e) {
	if constexpr (requires { EditorLowering<E>::LowerColor(e); }) {
		return EditorLowering<E>::LowerColor(e);
	} else if constexpr (DeviceColorEditor<E>) {
		constexpr int mode = detail::ModeOf<E>::value;
		static_assert(mode == -1 || mode == 0 || mode == 2, "colour edits fill or paint (a dig is a geometry edit)");
		hd_vbr_edit_desc d{};
		d.edit = detail::lower_shape(e, mode == 2 ? HD_OP_PAINT : HD_OP_FILL);
		d.colors = (uint32_t)e.color.GetColors();
		d.weight = (uint32_t)e.color.GetWeight();
		d.bits_per_weight = (uint32_t)e.color.GetBitsPerWeight();
		return d;
	} else {
		static_assert(detail::kAlwaysFalse<E>, "not a colour editor the device can apply");
		return {};
	}
}

class GpuNodePool {
public:
	/* DAGNodePool::Create (src/DAGNodePool.cpp:9-47): the pool, or nullptr
	 * (reason in *status).  heap_pages 0 = one device page per virtual page
	 * (identity heap); index_log2 0 = index sized from the heap. */
	static std::unique_ptr<GpuNodePool> Create(const hd_config &config, uint64_t heap_pages = 0, int device = 0,
	                                           hd_status *status = nullptr, uint32_t index_log2 = 0) {
		hd_pool *p = nullptr;
		const uint64_t heap = heap_pages ? heap_pages : (uint64_t)config_total_pages(config);
		const hd_status s = hd_pool_create(&config, heap, index_log2, device, &p);
		if (status)
			*status = s;
		if (s != HD_OK)
			return nullptr;
		return std::unique_ptr<GpuNodePool>(new GpuNodePool(p, config));
	}
	~GpuNodePool() { hd_pool_destroy(m_pool); }
	GpuNodePool(const GpuNodePool &) = delete;
	GpuNodePool &operator=(const GpuNodePool &) = delete;

	hd_pool *Handle() const { return m_pool; }
	const hd_config &GetHdConfig() const { return m_mirror.MirrorConfig(); }

	/* NodePoolBase::Edit / NodePoolThreadedEdit::ThreadedEdit
	 * (include/hashdag/NodePool.hpp:405-417, NodePoolThreadedEdit.hpp:104-126)
	 * for stateless sphere / box editors: edits applied in order, one pass on
	 * the device.  On failure *new_root keeps root. */
	hd_status Edit(uint32_t root, std::span<const hd_edit_desc> edits, uint32_t *new_root, void *stream = nullptr) {
		return hd_edit(m_pool, root, edits.data(), (uint32_t)edits.size(), new_root, stream);
	}
	/* The same for the reference's editor objects (lowered by LowerEditor):
	 * one editor, or a span of editors of one type applied in order in one
	 * batched pass. */
	template <DeviceEditor E>
	hd_status Edit(uint32_t root, const E &editor, uint32_t *new_root, void *stream = nullptr) {
		const hd_edit_desc d = LowerEditor(editor);
		return hd_edit(m_pool, root, &d, 1u, new_root, stream);
	}
	template <DeviceEditor E>
	hd_status Edit(uint32_t root, std::span<const E> editors, uint32_t *new_root, void *stream = nullptr) {
		std::vector<hd_edit_desc> d;
		d.reserve(editors.size());
		for (const E &e : editors)
			d.push_back(LowerEditor(e));
		return hd_edit(m_pool, root, d.data(), (uint32_t)d.size(), new_root, stream);
	}
	/* The reference's own call forms, root in and root out: NodePoolBase::Edit
	 * (NodePool.hpp:405-417) and NodePoolThreadedEdit::ThreadedEdit
	 * (NodePoolThreadedEdit.hpp:104-126, as src/main.cpp:214-223 calls it).
	 * The task pool and max_task_level only schedule the reference's CPU
	 * recursion; the device pass takes their place and ignores them.  On
	 * failure the old root comes back and LastStatus() says why. */
	template <DeviceEditor E> uint32_t Edit(uint32_t root, const E &editor) {
		uint32_t r = root;
		m_last_status = Edit(root, editor, &r);
		return m_last_status == HD_OK ? r : root;
	}
	template <class TaskPool, DeviceEditor E>
	uint32_t ThreadedEdit(TaskPool * /*busy_pool*/, uint32_t root, const E &editor, uint32_t /*max_task_level*/) {
		return Edit(root, editor);
	}
	hd_status LastStatus() const { return m_last_status; }
	/* NodePoolThreadedGC::ThreadedGC (NodePoolThreadedGC.hpp:394-403): roots
	 * remapped in place; the mirror is stale afterwards (the next Publish
	 * reads everything). */
	hd_status GC(std::span<uint32_t> roots, hd_gc_stats *stats = nullptr) {
		return hd_gc(m_pool, roots.data(), (uint32_t)roots.size(), stats);
	}
	/* m_filled_node_pointers (NodePool.hpp:54), one per level. */
	hd_status FilledPointers(std::vector<uint32_t> *out) const {
		out->assign(GetHdConfig().node_levels, HD_NULL_PTR);
		return hd_pool_filled_pointers(m_pool, out->data());
	}
	/* SetRoot / GetRoot (src/DAGNodePool.hpp:96-97): the root the renderer traces. */
	void SetRoot(uint32_t root) { m_root = root; }
	uint32_t GetRoot() const { return m_root; }

	/* ---- host mirror */
	HostPoolMirror &Mirror() { return m_mirror; }
	const HostPoolMirror &Mirror() const { return m_mirror; }
	/* Device -> mirror: every bucket's word count and every page that holds
	 * data (the words the reference's hooks would hold); the mirror's other
	 * pages are dropped and nothing is marked dirty.  Waits for the pool's
	 * queued passes. */
	hd_status Download() {
		HostPoolMirror &m = m_mirror;
		uint64_t epoch = 0;
		hd_status s = hd_pool_epoch(m_pool, &epoch);
		if (s != HD_OK)
			return s;
		m_synced = false;
		std::vector<uint32_t> counts(m.TotalBuckets());
		if ((s = hd_pool_read_bucket_words(m_pool, 0, m.TotalBuckets(), counts.data())) != HD_OK)
			return s;
		std::vector<uint8_t> map(m.TotalPages());
		if ((s = hd_pool_read_page_map(m_pool, map.data())) != HD_OK)
			return s;
		std::vector<uint32_t> ids;
		for (uint32_t i = 0; i < m.TotalPages(); ++i)
			if (map[i])
				ids.push_back(i);
		m.Clear();
		for (uint32_t b = 0; b < m.TotalBuckets(); ++b)
			m.GetBucketRefWords(b) = counts[b];
		const uint32_t wpp = m.WordsPerPage();
		const uint32_t chunk = kChunkWords / wpp ? kChunkWords / wpp : 1u;
		std::vector<uint32_t> words((size_t)chunk * wpp);
		for (size_t first = 0; first < ids.size(); first += chunk) {
			const uint32_t n = (uint32_t)std::min<size_t>(chunk, ids.size() - first);
			if ((s = hd_pool_read_pages(m_pool, ids.data() + first, n, words.data())) != HD_OK)
				return s;
			for (uint32_t k = 0; k < n; ++k)
				m.SetPage(ids[first + k], words.data() + (size_t)k * wpp);
		}
		m_epoch = epoch;
		m_synced = true;
		return HD_OK;
	}
	/* Device -> mirror, only what changed: the dirty-range publish of the
	 * application's pool (src/DAGNodePool.hpp:62-69, Flush in
	 * src/DAGNodePool.cpp:56-85).  While the pool's epoch (hd_pool_epoch) is
	 * the one of the mirror's last sync the pool only appended, so only the
	 * pages covering each bucket's new words are read, and those words become
	 * the pages' written ranges.  After a GC, rollback or upload (a new epoch),
	 * or before the first sync, everything is read: each page the pool holds
	 * then counts as written in full and each page it no longer holds as
	 * freed.  Dirty state accumulates until ClearDirty.  *full (may be NULL)
	 * tells which form ran.  No other thread may rewrite the pool meanwhile. */
	hd_status Publish(bool *full = nullptr) {
		HostPoolMirror &m = m_mirror;
		uint64_t epoch = 0;
		hd_status s = hd_pool_epoch(m_pool, &epoch);
		if (s != HD_OK)
			return s;
		std::vector<uint32_t> counts(m.TotalBuckets());
		std::vector<AppendedPage> pages;
		bool incremental = m_synced && epoch == m_epoch;
		if (incremental) {
			if ((s = hd_pool_read_bucket_words(m_pool, 0, m.TotalBuckets(), counts.data())) != HD_OK)
				return s;
			incremental = m.AppendedPages(counts, &pages);
		}
		if (full)
			*full = !incremental;
		if (!incremental)
			return publish_all();
		const uint32_t wpp = m.WordsPerPage();
		const uint32_t chunk = kChunkWords / wpp ? kChunkWords / wpp : 1u;
		std::vector<uint32_t> ids, words((size_t)chunk * wpp);
		for (size_t first = 0; first < pages.size(); first += chunk) {
			const uint32_t n = (uint32_t)std::min<size_t>(chunk, pages.size() - first);
			ids.clear();
			for (uint32_t k = 0; k < n; ++k)
				ids.push_back(pages[first + k].page_id);
			if ((s = hd_pool_read_pages(m_pool, ids.data(), n, words.data())) != HD_OK)
				return s;
			for (uint32_t k = 0; k < n; ++k) {
				const PageRange r = pages[first + k].words;
				m.WritePage(ids[k], r.begin,
				            std::span<const uint32_t>(words.data() + (size_t)k * wpp + r.begin, r.end - r.begin));
			}
		}
		for (uint32_t b = 0; b < m.TotalBuckets(); ++b)
			m.GetBucketRefWords(b) = counts[b];
		uint64_t after = 0;
		if ((s = hd_pool_epoch(m_pool, &after)) != HD_OK)
			return s;
		if (after != epoch) { // rewritten while it was read
			if (full)
				*full = true;
			return publish_all();
		}
		return HD_OK;
	}
	/* Mirror -> device: replaces the device pool with the mirror's words
	 * (bucket counts and every page that holds data), rebuilds the dedup index
	 * and finds the filled nodes again (appending them if the mirror lacks
	 * them; the mirror then receives those words as written ranges, else it is
	 * clean afterwards).  Roots made on the device before the call are valid
	 * only if the mirror holds their nodes. */
	hd_status Upload() {
		HostPoolMirror &m = m_mirror;
		const std::vector<uint32_t> ids = m.PageIds();
		const uint32_t wpp = m.WordsPerPage();
		std::vector<uint32_t> words(ids.size() * (size_t)wpp);
		for (size_t k = 0; k < ids.size(); ++k)
			std::copy(m.ReadPage(ids[k]), m.ReadPage(ids[k]) + wpp, words.data() + k * wpp);
		hd_status s = hd_pool_upload(m_pool, m.BucketWords().data(), ids.data(), (uint32_t)ids.size(), words.data(),
		                             nullptr);
		m_synced = false;
		if (s != HD_OK)
			return s;
		m.ClearDirty();
		// the upload found or inserted the filled nodes: bring their words over
		uint64_t epoch = 0;
		if ((s = hd_pool_epoch(m_pool, &epoch)) != HD_OK)
			return s;
		m_epoch = epoch;
		m_synced = true;
		return Publish();
	}

	/* The reference's storage hooks, on the mirror (NodePool.hpp:22-38). */
	uint32_t &GetBucketRefWords(uint32_t bucket_id) { return m_mirror.GetBucketRefWords(bucket_id); }
	const uint32_t *ReadPage(uint32_t page_id) const { return m_mirror.ReadPage(page_id); }
	void ZeroPage(uint32_t page_id, uint32_t page_offset, uint32_t zero_words) {
		m_mirror.ZeroPage(page_id, page_offset, zero_words);
	}
	void WritePage(uint32_t page_id, uint32_t page_offset, std::span<const uint32_t> word_span) {
		m_mirror.WritePage(page_id, page_offset, word_span);
	}
	std::mutex &GetBucketRefMutex(uint32_t bucket_id) { return m_mirror.GetBucketRefMutex(bucket_id); }
	void FreePage(uint32_t page_id) { m_mirror.FreePage(page_id); }

private:
	static constexpr uint32_t kChunkWords = 1u << 24; // 64 MB of page words per read

	hd_status publish_all() {
		HostPoolMirror &m = m_mirror;
		std::vector<uint8_t> had(m.TotalPages());
		for (uint32_t i = 0; i < m.TotalPages(); ++i)
			had[i] = m.HasPage(i) || m.IsFreed(i);
		const hd_status s = Download();
		if (s != HD_OK)
			return s;
		for (uint32_t i = 0; i < m.TotalPages(); ++i) {
			if (m.HasPage(i))
				m.MarkWritten(i, PageRange{0u, m.WordsPerPage()});
			else if (had[i])
				m.FreePage(i);
		}
		return HD_OK;
	}

	GpuNodePool(hd_pool *pool, const hd_config &config) : m_pool(pool), m_mirror(config) {}

	hd_pool *m_pool;
	HostPoolMirror m_mirror;
	uint32_t m_root = HD_NULL_PTR;
	hd_status m_last_status = HD_OK;
	uint64_t m_epoch = 0; // hd_pool_epoch at the mirror's last full or incremental sync
	bool m_synced = false;
};

/* The application's colour octree DAGColorPool (src/DAGColorPool.hpp:20-218)
 * on the device, for the voxels of one GpuNodePool, edited with it as the
 * application's vbr_edit lambda does (src/main.cpp:224-242: Edit with a
 * VBREditorWrapper, then set_root of both roots).  Destroy it before its
 * node pool. */
class GpuColorPool {
public:
	static constexpr uint32_t kNull = HD_COLOR_NULL;

	/* DAGColorPool::Create (src/DAGColorPool.cpp:9-47, Config leaf_level and
	 * keep_history): the pool, or nullptr (reason in *status). */
	static std::unique_ptr<GpuColorPool> Create(GpuNodePool &nodes, uint32_t leaf_level, bool keep_history = false,
	                                            uint64_t max_nodes = uint64_t(1) << 20,
	                                            uint64_t max_leaf_words = uint64_t(1) << 24, hd_status *status = nullptr) {
		hd_color_config c{};
		c.leaf_level = leaf_level;
		c.keep_history = keep_history ? 1u : 0u;
		c.max_nodes = max_nodes;
		c.max_leaf_words = max_leaf_words;
		hd_color_pool *p = nullptr;
		const hd_status s = hd_color_pool_create(nodes.Handle(), &c, &p);
		if (status)
			*status = s;
		if (s != HD_OK)
			return nullptr;
		return std::unique_ptr<GpuColorPool>(new GpuColorPool(nodes, p, leaf_level));
	}
	~GpuColorPool() { hd_color_pool_destroy(m_pool); }
	GpuColorPool(const GpuColorPool &) = delete;
	GpuColorPool &operator=(const GpuColorPool &) = delete;

	hd_color_pool *Handle() const { return m_pool; }
	uint32_t GetLeafLevel() const { return m_leaf_level; }
	/* SetRoot / GetRoot (src/DAGColorPool.hpp) */
	void SetRoot(uint32_t color_root) { m_root = color_root; }
	uint32_t GetRoot() const { return m_root; }

	/* Colour edits in order from the node pool's and this pool's roots; on
	 * success both roots are set (set_root of src/main.cpp:239-243).  A full
	 * octree fails the edit that overflowed it, with both roots as after the
	 * edit before. */
	hd_status VbrEdit(std::span<const hd_vbr_edit_desc> edits) {
		uint32_t root = m_nodes.GetRoot(), color_root = m_root;
		const hd_status s = hd_vbr_edit(m_nodes.Handle(), m_pool, root, color_root, edits.data(),
		                                (uint32_t)edits.size(), &root, &color_root);
		if (s == HD_OK || s == HD_ERR_POOL_OOM) {
			m_nodes.SetRoot(root);
			m_root = color_root;
		}
		return s;
	}
	/* The application's colour editor objects (VBREditorWrapper over
	 * SphereEditor<kFill / kPaint> or AABBEditor with their VBRColor,
	 * src/main.cpp:224-242), lowered by LowerColorEditor. */
	template <DeviceColorEditor E> hd_status VbrEdit(const E &editor) {
		const hd_vbr_edit_desc d = LowerColorEditor(editor);
		return VbrEdit(std::span<const hd_vbr_edit_desc>(&d, 1));
	}
	/* The host mirror: the node and leaf word vectors of DAGColorPool, the
	 * words its Flush uploads (src/DAGColorPool.cpp:49-80). */
	hd_status Read(std::vector<uint32_t> *nodes, std::vector<uint32_t> *leaf_words) const {
		uint64_t nn = 0, nl = 0;
		hd_status s = hd_color_pool_read(m_pool, nullptr, &nn, nullptr, &nl);
		if (s != HD_OK)
			return s;
		nodes->resize(nn * 8);
		leaf_words->resize(nl);
		return hd_color_pool_read(m_pool, nodes->data(), &nn, leaf_words->data(), &nl);
	}
	/* Colours of n voxels under the current colour root (trace.frag Color_Fetch;
	 * device buffers). */
	hd_status Fetch(const uint32_t *d_xyz, uint32_t n, hd_vbr_color *d_out, void *stream = nullptr) const {
		return hd_color_fetch(m_pool, m_root, d_xyz, n, d_out, stream);
	}

private:
	GpuColorPool(GpuNodePool &nodes, hd_color_pool *pool, uint32_t leaf_level)
	    : m_nodes(nodes), m_pool(pool), m_leaf_level(leaf_level) {}

	GpuNodePool &m_nodes;
	hd_color_pool *m_pool;
	uint32_t m_leaf_level;
	uint32_t m_root = kNull;
};

} // namespace hashdag_gb300
