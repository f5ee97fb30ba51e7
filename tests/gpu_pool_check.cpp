// gpu_pool_check.cpp -- checks of the C++ host side of the pool
// (include/hashdag_gpu_pool.hpp, include/hashdag_host_mirror.hpp), built by
// tests/test_cpp_pool.py.
//
// Linked against libhashdag_gb300.so:
//   gpu_pool_check mirror    HostPoolMirror's storage hooks and bookkeeping
//   gpu_pool_check nodevice  GpuNodePool::Create with no usable device:
//                            nullptr and HD_ERR_NO_DEVICE, like DAGNodePool::Create
//   gpu_pool_check device    on a GPU: edits on the device, Download into the
//                            mirror, Upload of that mirror into a second pool
//                            (word for word the same pool, same filled
//                            pointers), the same further edits on both, and
//                            occupancy against the edits' own predicates;
//                            then GC through the class and the same check
//   gpu_pool_check publish   on a GPU: incremental Publish after edits equals a
//                            full Download; after a GC it re-reads everything
//   gpu_pool_check color     on a GPU: GpuColorPool, the same colour edits one
//                            per call and in one call give the same octree words
//   gpu_pool_check editors EDITS DUMP  on a GPU: the hd_edit_desc records in
//                            file EDITS as the application's editor objects
//                            (SphereEditor<kFill/kDig>, AABBEditor, a box dig),
//                            applied one per call through the reference's call
//                            forms (ThreadedEdit(&busy_pool, root, editor, mtl)
//                            and Edit(root, editor)), against one batched pass
//                            of the descriptors; the pool is saved to DUMP and
//                            "root R" printed for the caller's canonical check
// Built with -DHD_FAKE_DEVICE instead (no library, no GPU): the pool entry
// points GpuNodePool calls are served by an in-memory pool below, and
//   gpu_pool_check fake_publish   Publish: full on the first sync and after an
//                                 epoch change (freed pages reported), else
//                                 only the appended words, as written ranges
//   gpu_pool_check dump           Save / Load of a pool dump
//   gpu_pool_check dump_copy IN OUT   Load IN, Save OUT (format round trips)
//   gpu_pool_check lowering       LowerEditor / LowerColorEditor of the
//                                 application's editor layouts
// Prints "ok <mode>" and exits 0, or prints the first failure and exits 1.
#include "hashdag_gpu_pool.hpp"

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using hashdag_gb300::GpuNodePool;
using hashdag_gb300::HostPoolMirror;

#define CHECK(c)                                                                                                      \
	do {                                                                                                              \
		if (!(c)) {                                                                                                   \
			std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);                                                \
			return 1;                                                                                                 \
		}                                                                                                             \
	} while (0)
#define CHECK_OK(s)                                                                                                   \
	do {                                                                                                              \
		const hd_status s_ = (s);                                                                                     \
		if (s_ != HD_OK) {                                                                                            \
			std::printf("FAILED %s:%d: %s -> %s\n", __FILE__, __LINE__, #s, hd_status_string(s_));                    \
			return 1;                                                                                                 \
		}                                                                                                             \
	} while (0)

#ifdef HD_FAKE_DEVICE
// DefaultConfig for a 256^3 grid written out (hd_config_default lives in the library)
static hd_config small_config() {
	hd_config c{};
	c.word_bits_per_page = 9;
	c.page_bits_per_bucket = 2;
	c.node_levels = 7;
	c.hasher = HD_HASHER_MURMUR32;
	for (uint32_t l = 0; l < 7; ++l)
		c.bucket_bits_each_level[l] = 10;
	return c;
}

// The pool entry points GpuNodePool calls, on an in-memory pool: its words in
// a HostPoolMirror and the epoch the library keeps (hd_pool_epoch).
struct hd_pool {
	explicit hd_pool(const hd_config &c) : words(c) {}
	HostPoolMirror words;
	uint64_t epoch = 0;
};
extern "C" {
hd_status hd_pool_create(const hd_config *config, uint64_t, uint32_t, int, hd_pool **out) {
	*out = new hd_pool(*config);
	return HD_OK;
}
void hd_pool_destroy(hd_pool *p) { delete p; }
hd_status hd_pool_epoch(const hd_pool *p, uint64_t *out) {
	*out = p->epoch;
	return HD_OK;
}
hd_status hd_pool_read_bucket_words(const hd_pool *p, uint32_t first, uint32_t count, uint32_t *out) {
	if ((uint64_t)first + count > p->words.TotalBuckets())
		return HD_ERR_INVALID_ARG;
	std::copy(p->words.BucketWords().begin() + first, p->words.BucketWords().begin() + first + count, out);
	return HD_OK;
}
hd_status hd_pool_read_page_map(const hd_pool *p, uint8_t *out) {
	for (uint32_t i = 0; i < p->words.TotalPages(); ++i)
		out[i] = p->words.HasPage(i) ? 1 : 0;
	return HD_OK;
}
hd_status hd_pool_read_pages(const hd_pool *p, const uint32_t *ids, uint32_t n, uint32_t *out) {
	const uint32_t wpp = p->words.WordsPerPage();
	for (uint32_t k = 0; k < n; ++k) {
		if (ids[k] >= p->words.TotalPages())
			return HD_ERR_INVALID_ARG;
		const uint32_t *w = p->words.ReadPage(ids[k]);
		for (uint32_t i = 0; i < wpp; ++i)
			out[(size_t)k * wpp + i] = w ? w[i] : 0u; // an unmapped page reads as zeros
	}
	return HD_OK;
}
hd_status hd_pool_upload(hd_pool *p, const uint32_t *bucket_words, const uint32_t *ids, uint32_t n,
                         const uint32_t *page_words, const uint32_t *) {
	++p->epoch;
	p->words.Clear();
	for (uint32_t b = 0; b < p->words.TotalBuckets(); ++b)
		p->words.GetBucketRefWords(b) = bucket_words[b];
	for (uint32_t k = 0; k < n; ++k)
		p->words.SetPage(ids[k], page_words + (size_t)k * p->words.WordsPerPage());
	return HD_OK;
}
const char *hd_status_string(hd_status) { return "status"; }
}
#else
static hd_config small_config() {
	hd_config c;
	// DefaultConfig for a 256^3 grid: level_count 8, 9 top levels of 2^10
	// buckets (so every one of the 7 node levels), 512-word pages, 4 per bucket
	hd_config_default(8, 9, 9, 2, 10, 16, &c);
	return c;
}
#endif

// The application's editor objects (src/main.cpp:32-150), restated with their
// member names and template shape: glm::u32vec3 fields, an EditMode template
// argument, and a colour with VBRColor's accessors
// (include/hashdag/VBRColor.hpp:18-43).  Their EditNode / EditVoxel run only in
// the reference's CPU recursion; the device lowers the objects to descriptors.
namespace app {
struct u32vec3 {
	uint32_t x, y, z;
};
enum class EditMode { kFill, kDig, kPaint };
class VBRColor {
public:
	constexpr VBRColor() = default;
	constexpr VBRColor(uint32_t colors, uint8_t weight, uint8_t bpw)
	    : m_colors(colors), m_weight(weight), m_bits_per_weight(bpw), m_has_value(true) {}
	constexpr uint32_t GetColors() const { return m_colors; }
	constexpr uint8_t GetWeight() const { return m_weight; }
	constexpr uint8_t GetBitsPerWeight() const { return m_bits_per_weight; }
	constexpr bool HasValue() const { return m_has_value; }

private:
	uint32_t m_colors{};
	uint8_t m_weight{}, m_bits_per_weight{};
	bool m_has_value{false};
};
struct AABBEditor {
	u32vec3 aabb_min, aabb_max;
	VBRColor color;
};
template <EditMode Mode = EditMode::kFill> struct SphereEditor {
	u32vec3 center{};
	uint64_t r2{};
	VBRColor color;
};
// the box dig of the benchmark's workloads (the application's AABBEditor fills only)
template <EditMode Mode> struct BoxEditor {
	u32vec3 aabb_min, aabb_max;
};
struct BusyPool {}; // stands for lf::busy_pool: the device pass ignores it
} // namespace app

static_assert(hashdag_gb300::DeviceEditor<app::AABBEditor>);
static_assert(hashdag_gb300::DeviceEditor<app::SphereEditor<app::EditMode::kFill>>);
static_assert(hashdag_gb300::DeviceEditor<app::SphereEditor<app::EditMode::kDig>>);
static_assert(!hashdag_gb300::DeviceEditor<app::SphereEditor<app::EditMode::kPaint>>); // colours only
static_assert(hashdag_gb300::DeviceEditor<app::BoxEditor<app::EditMode::kDig>>);
static_assert(!hashdag_gb300::DeviceEditor<hd_edit_desc> && !hashdag_gb300::DeviceEditor<int>);
static_assert(hashdag_gb300::DeviceColorEditor<app::SphereEditor<app::EditMode::kPaint>>);
static_assert(hashdag_gb300::DeviceColorEditor<app::AABBEditor>);
static_assert(!hashdag_gb300::DeviceColorEditor<app::BoxEditor<app::EditMode::kDig>>); // no colour

[[maybe_unused]] static bool same_desc(const hd_edit_desc &a, const hd_edit_desc &b) {
	return a.shape == b.shape && a.op == b.op && a.r2 == b.r2 && std::memcmp(a.p0, b.p0, 12) == 0 &&
	       std::memcmp(a.p1, b.p1, 12) == 0;
}

static int check_lowering() {
	using namespace app;
	const hd_edit_desc s = hashdag_gb300::LowerEditor(SphereEditor<EditMode::kDig>{{7, 8, 9}, 400, {}});
	CHECK(s.shape == HD_SHAPE_SPHERE && s.op == HD_OP_DIG && s.p0[0] == 7 && s.p0[1] == 8 && s.p0[2] == 9 &&
	      s.r2 == 400 && s.p1[0] == 0);
	const hd_edit_desc f = hashdag_gb300::LowerEditor(SphereEditor<>{{1, 2, 3}, 25, {}});
	CHECK(f.shape == HD_SHAPE_SPHERE && f.op == HD_OP_FILL && f.r2 == 25);
	const hd_edit_desc b = hashdag_gb300::LowerEditor(AABBEditor{{1, 2, 3}, {4, 5, 6}, {}});
	CHECK(b.shape == HD_SHAPE_AABB && b.op == HD_OP_FILL && b.p0[2] == 3 && b.p1[0] == 4 && b.p1[2] == 6 && b.r2 == 0);
	const hd_edit_desc d = hashdag_gb300::LowerEditor(BoxEditor<EditMode::kDig>{{0, 0, 0}, {64, 64, 64}});
	CHECK(d.shape == HD_SHAPE_AABB && d.op == HD_OP_DIG && d.p1[1] == 64);
	const hd_vbr_edit_desc p =
	    hashdag_gb300::LowerColorEditor(SphereEditor<EditMode::kPaint>{{5, 5, 5}, 9, VBRColor(0x123456u, 3, 2)});
	CHECK(p.edit.op == HD_OP_PAINT && p.edit.shape == HD_SHAPE_SPHERE && p.colors == 0x123456u && p.weight == 3 &&
	      p.bits_per_weight == 2);
	const hd_vbr_edit_desc c = hashdag_gb300::LowerColorEditor(AABBEditor{{1, 1, 1}, {2, 2, 2}, VBRColor(0xFFu, 0, 0)});
	CHECK(c.edit.op == HD_OP_FILL && c.edit.shape == HD_SHAPE_AABB && c.colors == 0xFFu && c.bits_per_weight == 0);
	return 0;
}

static bool same_mirror(const HostPoolMirror &a, const HostPoolMirror &b) {
	if (a.BucketWords() != b.BucketWords() || a.PageIds() != b.PageIds())
		return false;
	for (uint32_t id : a.PageIds())
		if (std::memcmp(a.ReadPage(id), b.ReadPage(id), a.WordsPerPage() * 4u) != 0)
			return false;
	return true;
}

static int check_mirror() {
	const hd_config c = small_config();
	HostPoolMirror m(c);
	CHECK(m.TotalBuckets() == 7u * 1024u && m.TotalPages() == m.TotalBuckets() * 4u && m.WordsPerPage() == 512u);
	CHECK(m.ReadPage(3) == nullptr && !m.HasPage(3) && m.PageIds().empty());
	const uint32_t w[3] = {11, 12, 13};
	m.WritePage(3, 5, std::span<const uint32_t>(w, 3));
	CHECK(m.HasPage(3) && m.IsDirty(3) && !m.IsDirty(4));
	const uint32_t *p = m.ReadPage(3);
	CHECK(p[4] == 0 && p[5] == 11 && p[6] == 12 && p[7] == 13 && p[8] == 0 && p[511] == 0);
	m.ZeroPage(3, 6, 1);
	CHECK(p[5] == 11 && p[6] == 0 && p[7] == 13);
	m.ZeroPage(9, 0, 4); // a page never written: created zeroed
	CHECK(m.HasPage(9) && m.ReadPage(9)[0] == 0 && m.IsDirty(9));
	m.GetBucketRefWords(2) = 17;
	CHECK(m.BucketWords()[2] == 17 && m.BucketWords()[1] == 0);
	CHECK((m.PageIds() == std::vector<uint32_t>{3, 9}));
	m.ClearDirty();
	CHECK(!m.IsDirty(3) && !m.IsDirty(9));
	m.FreePage(3);
	CHECK(!m.HasPage(3) && m.ReadPage(3) == nullptr && m.IsDirty(3));
	CHECK(&m.GetBucketRefMutex(5) == &m.GetBucketRefMutex(5 + 1024));
	m.GetBucketRefMutex(5).lock();
	CHECK(m.GetBucketRefMutex(6).try_lock());
	m.GetBucketRefMutex(6).unlock();
	m.GetBucketRefMutex(5).unlock();
	std::vector<uint32_t> words(512, 7);
	m.SetPage(20, words.data());
	CHECK(m.HasPage(20) && !m.IsDirty(20) && m.ReadPage(20)[511] == 7);
	m.Clear();
	CHECK(m.PageIds().empty() && m.BucketWords()[2] == 0);
	return 0;
}

#ifndef HD_FAKE_DEVICE
static int check_nodevice() {
	hd_status s = HD_OK;
	auto pool = GpuNodePool::Create(small_config(), 0, 0, &s);
	CHECK(pool == nullptr && s == HD_ERR_NO_DEVICE);
	hd_config bad = small_config();
	bad.word_bits_per_page = 40;
	pool = GpuNodePool::Create(bad, 0, 0, &s);
	CHECK(pool == nullptr && s == HD_ERR_INVALID_ARG);
	return 0;
}

static hd_edit_desc sphere(uint32_t op, uint32_t x, uint32_t y, uint32_t z, uint64_t r) {
	hd_edit_desc e{};
	e.shape = HD_SHAPE_SPHERE;
	e.op = op;
	e.p0[0] = x, e.p0[1] = y, e.p0[2] = z;
	e.r2 = r * r;
	return e;
}
static hd_edit_desc box(uint32_t op, uint32_t x0, uint32_t y0, uint32_t z0, uint32_t x1, uint32_t y1, uint32_t z1) {
	hd_edit_desc e{};
	e.shape = HD_SHAPE_AABB;
	e.op = op;
	e.p0[0] = x0, e.p0[1] = y0, e.p0[2] = z0;
	e.p1[0] = x1, e.p1[1] = y1, e.p1[2] = z1;
	return e;
}
// VoxelInRange of the stateless editors (src/main.cpp:55-57,121-126), applied in order.
static bool truth(const std::vector<hd_edit_desc> &edits, uint32_t x, uint32_t y, uint32_t z) {
	bool v = false;
	for (const hd_edit_desc &e : edits) {
		bool in;
		if (e.shape == HD_SHAPE_AABB) {
			in = x >= e.p0[0] && x < e.p1[0] && y >= e.p0[1] && y < e.p1[1] && z >= e.p0[2] && z < e.p1[2];
		} else {
			const long long dx = (long long)x - e.p0[0], dy = (long long)y - e.p0[1], dz = (long long)z - e.p0[2];
			in = (unsigned long long)(dx * dx + dy * dy + dz * dz) <= e.r2;
		}
		if (in)
			v = e.op == HD_OP_FILL;
	}
	return v;
}

static int check_occupancy(GpuNodePool &pool, uint32_t root, const std::vector<hd_edit_desc> &edits, int *set_out) {
	std::vector<uint32_t> xyz;
	uint64_t s = 0x2545F4914F6CDD1Dull;
	for (int i = 0; i < 1 << 15; ++i)
		for (int a = 0; a < 3; ++a) {
			s ^= s << 13, s ^= s >> 7, s ^= s << 17;
			xyz.push_back((uint32_t)(s >> 40) & 255u);
		}
	std::vector<uint8_t> out(xyz.size() / 3);
	CHECK_OK(hd_query(pool.Handle(), root, xyz.data(), (uint32_t)out.size(), out.data(), nullptr));
	int set = 0;
	for (size_t i = 0; i < out.size(); ++i) {
		const bool want = truth(edits, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
		if ((out[i] != 0) != want) {
			std::printf("FAILED occupancy at (%u,%u,%u): %d vs %d\n", xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2],
			            out[i], (int)want);
			return 1;
		}
		set += want;
	}
	*set_out = set;
	return 0;
}

static int check_device() {
	const hd_config c = small_config();
	hd_status s = HD_OK;
	auto a = GpuNodePool::Create(c, 0, 0, &s);
	CHECK_OK(s);
	CHECK(a != nullptr);
	std::vector<hd_edit_desc> edits = {sphere(HD_OP_FILL, 128, 128, 128, 70), box(HD_OP_FILL, 10, 20, 30, 90, 60, 250),
	                                   sphere(HD_OP_DIG, 150, 100, 140, 30), box(HD_OP_DIG, 0, 0, 0, 140, 128, 120),
	                                   sphere(HD_OP_FILL, 40, 200, 60, 25)};
	uint32_t root = HD_NULL_PTR;
	CHECK_OK(a->Edit(HD_NULL_PTR, edits, &root));
	a->SetRoot(root);
	CHECK(a->GetRoot() == root && root != HD_NULL_PTR);

	CHECK_OK(a->Download());
	const HostPoolMirror &ma = a->Mirror();
	uint64_t words = 0;
	for (uint32_t w : ma.BucketWords())
		words += w;
	CHECK(words > 0 && !ma.PageIds().empty());
	for (uint32_t id : ma.PageIds())
		CHECK(!ma.IsDirty(id) && a->ReadPage(id) == ma.ReadPage(id));
	// the words of the root node, read through the reference's hook
	const uint32_t *rootw = a->ReadPage(root >> c.word_bits_per_page) + (root & ((1u << c.word_bits_per_page) - 1u));
	CHECK((rootw[0] & 0xFFu) != 0);

	// a second pool built from the first one's mirror
	auto b = GpuNodePool::Create(c, 0, 0, &s);
	CHECK_OK(s);
	for (uint32_t i = 0; i < ma.TotalBuckets(); ++i)
		b->GetBucketRefWords(i) = ma.BucketWords()[i];
	for (uint32_t id : ma.PageIds())
		b->WritePage(id, 0, std::span<const uint32_t>(ma.ReadPage(id), ma.WordsPerPage()));
	CHECK(b->Mirror().IsDirty(ma.PageIds()[0]));
	CHECK_OK(b->Upload());
	CHECK(!b->Mirror().IsDirty(ma.PageIds()[0]));
	CHECK_OK(b->Download());
	CHECK(same_mirror(ma, b->Mirror()));
	std::vector<uint32_t> fa, fb;
	CHECK_OK(a->FilledPointers(&fa));
	CHECK_OK(b->FilledPointers(&fb));
	CHECK(fa == fb);

	// the same further edits on both pools from the same root
	const std::vector<hd_edit_desc> more = {sphere(HD_OP_DIG, 128, 128, 128, 20), box(HD_OP_FILL, 200, 0, 0, 256, 40, 256),
	                                        sphere(HD_OP_FILL, 60, 60, 200, 45)};
	uint32_t ra = HD_NULL_PTR, rb = HD_NULL_PTR;
	CHECK_OK(a->Edit(root, more, &ra));
	CHECK_OK(b->Edit(root, more, &rb));
	std::vector<hd_edit_desc> all = edits;
	all.insert(all.end(), more.begin(), more.end());
	int set_a = 0, set_b = 0, set0 = 0;
	if (check_occupancy(*a, root, edits, &set0) || check_occupancy(*a, ra, all, &set_a) ||
	    check_occupancy(*b, rb, all, &set_b))
		return 1;
	CHECK(set0 > 1000 && set_a > 1000 && set_a == set_b);

	// GC through the class keeps the occupancy of the kept root
	uint32_t keep[1] = {ra};
	hd_gc_stats st{};
	CHECK_OK(a->GC(std::span<uint32_t>(keep, 1), &st));
	CHECK(st.live_nodes > 0 && st.words_after <= st.words_before);
	if (check_occupancy(*a, keep[0], all, &set_a))
		return 1;
	CHECK_OK(a->Download());
	uint64_t words_after = 0;
	for (uint32_t w : a->Mirror().BucketWords())
		words_after += w;
	CHECK(words_after == st.words_after);
	return 0;
}


// Incremental publish on a device that only appended: after one Publish, the
// real-device form must give the mirror a full Download gives, and a GC makes
// the next Publish read everything.
static int check_publish() {
	const hd_config c = small_config();
	hd_status s = HD_OK;
	auto a = GpuNodePool::Create(c, 0, 0, &s);
	CHECK_OK(s);
	bool full = false;
	CHECK_OK(a->Publish(&full));
	CHECK(full);
	uint32_t root = HD_NULL_PTR;
	const std::vector<hd_edit_desc> e1 = {sphere(HD_OP_FILL, 128, 128, 128, 60), box(HD_OP_DIG, 100, 0, 0, 256, 140, 256)};
	CHECK_OK(a->Edit(HD_NULL_PTR, e1, &root));
	a->Mirror().ClearDirty();
	CHECK_OK(a->Publish(&full));
	CHECK(!full);
	uint32_t dirty = 0;
	for (uint32_t id = 0; id < a->Mirror().TotalPages(); ++id)
		dirty += a->Mirror().IsDirty(id) ? 1u : 0u;
	CHECK(dirty > 0);
	const std::vector<hd_edit_desc> e2 = {sphere(HD_OP_DIG, 90, 160, 100, 40), box(HD_OP_FILL, 0, 0, 0, 60, 250, 30)};
	uint32_t root2 = HD_NULL_PTR;
	CHECK_OK(a->Edit(root, e2, &root2));
	CHECK_OK(a->Publish(&full));
	CHECK(!full);
	// the same words as a full read of the device
	HostPoolMirror &m = a->Mirror();
	std::vector<uint32_t> counts(m.TotalBuckets());
	CHECK_OK(hd_pool_read_bucket_words(a->Handle(), 0, m.TotalBuckets(), counts.data()));
	CHECK(counts == m.BucketWords());
	std::vector<uint8_t> map(m.TotalPages());
	CHECK_OK(hd_pool_read_page_map(a->Handle(), map.data()));
	std::vector<uint32_t> words(m.WordsPerPage());
	for (uint32_t id = 0; id < m.TotalPages(); ++id) {
		CHECK((map[id] != 0) == m.HasPage(id));
		if (!map[id])
			continue;
		CHECK_OK(hd_pool_read_pages(a->Handle(), &id, 1, words.data()));
		CHECK(std::memcmp(words.data(), m.ReadPage(id), m.WordsPerPage() * 4u) == 0);
	}
	// a collection rewrites: the next Publish reads everything
	uint32_t keep[1] = {root2};
	CHECK_OK(a->GC(std::span<uint32_t>(keep, 1)));
	m.ClearDirty();
	CHECK_OK(a->Publish(&full));
	CHECK(full);
	CHECK_OK(hd_pool_read_bucket_words(a->Handle(), 0, m.TotalBuckets(), counts.data()));
	CHECK(counts == m.BucketWords());
	return 0;
}

// GpuColorPool: the same coloured edits applied one per call and all in one
// call leave the same octree words and roots; digs keep the colour root.
static int color_run(bool one_call, std::vector<uint32_t> *nodes, std::vector<uint32_t> *leaves, uint32_t *croot) {
	const hd_config c = small_config();
	hd_status s = HD_OK;
	auto pool = GpuNodePool::Create(c, 0, 0, &s);
	CHECK_OK(s);
	auto colors = hashdag_gb300::GpuColorPool::Create(*pool, 3, false, 1u << 16, 1u << 22, &s);
	CHECK_OK(s);
	CHECK(colors != nullptr && colors->GetRoot() == HD_COLOR_NULL && colors->GetLeafLevel() == 3);
	std::vector<hd_vbr_edit_desc> v(6);
	const hd_edit_desc g[6] = {box(HD_OP_FILL, 10, 10, 10, 200, 120, 200), sphere(HD_OP_FILL, 128, 120, 100, 40),
	                           sphere(HD_OP_PAINT, 100, 100, 100, 30), box(HD_OP_DIG, 0, 0, 0, 60, 60, 60),
	                           sphere(HD_OP_FILL, 60, 60, 60, 20), sphere(HD_OP_PAINT, 180, 110, 150, 25)};
	for (int i = 0; i < 6; ++i) {
		v[i] = hd_vbr_edit_desc{};
		v[i].edit = g[i];
		v[i].colors = 0x102030u * uint32_t(i + 1);
	}
	v[2].bits_per_weight = 2; // a weighted paint: two R5G6B5 end points
	v[2].weight = 3;
	v[2].colors = 0x001F07E0u;
	if (one_call) {
		CHECK_OK(colors->VbrEdit(v));
	} else {
		for (size_t i = 0; i < v.size(); ++i) {
			const uint32_t before = colors->GetRoot();
			CHECK_OK(colors->VbrEdit(std::span<const hd_vbr_edit_desc>(v.data() + i, 1)));
			if (v[i].edit.op == HD_OP_DIG)
				CHECK(colors->GetRoot() == before);
		}
	}
	CHECK(pool->GetRoot() != HD_NULL_PTR && colors->GetRoot() != HD_COLOR_NULL);
	CHECK_OK(colors->Read(nodes, leaves));
	CHECK(!nodes->empty() && !leaves->empty() && nodes->size() % 8 == 0);
	*croot = colors->GetRoot();
	return 0;
}
static int check_color() {
	std::vector<uint32_t> n1, l1, n2, l2;
	uint32_t r1 = 0, r2 = 0;
	if (color_run(false, &n1, &l1, &r1) || color_run(true, &n2, &l2, &r2))
		return 1;
	CHECK(r1 == r2 && n1 == n2 && l1 == l2);
	return 0;
}
#else
static uint64_t g_rng = 0x9E3779B97F4A7C15ull;
static uint32_t rnd(uint32_t n) {
	g_rng ^= g_rng << 13, g_rng ^= g_rng >> 7, g_rng ^= g_rng << 17;
	return (uint32_t)(g_rng >> 32) % n;
}

// Appends a node of n words to bucket b the way upsert_node does
// (include/hashdag/NodePool.hpp:159-212): a node that would straddle a page
// starts on the next one (the skipped tail stays zero).
static bool append_node(HostPoolMirror &m, uint32_t b, uint32_t n) {
	const hd_config &c = m.MirrorConfig();
	const uint32_t wpp = m.WordsPerPage(), wpb = wpp << c.page_bits_per_bucket;
	uint32_t at = m.GetBucketRefWords(b);
	if ((at & (wpp - 1u)) + n > wpp)
		at = (at + wpp - 1u) & ~(wpp - 1u);
	if (at + n > wpb)
		return false;
	std::vector<uint32_t> w(n);
	for (auto &x : w)
		x = 1u + rnd(0xFFFFFFF0u);
	m.WritePage((b << c.page_bits_per_bucket) | (at >> c.word_bits_per_page), at & (wpp - 1u), w);
	m.GetBucketRefWords(b) = at + n;
	return true;
}
static void append_nodes(HostPoolMirror &m, int count, uint32_t buckets) {
	for (int i = 0; i < count; ++i)
		append_node(m, rnd(buckets), 2u + rnd(8));
}

// Publish against the in-memory pool: the first sync and every epoch change
// read everything (present pages written in full, vanished pages freed);
// otherwise exactly the words appended since, as each page's written range.
static int check_fake_publish() {
	const hd_config c = small_config();
	auto pool = GpuNodePool::Create(c);
	CHECK(pool != nullptr);
	hd_pool *dev = pool->Handle();
	HostPoolMirror &m = pool->Mirror();
	const uint32_t wpp = m.WordsPerPage();
	append_nodes(dev->words, 3000, 64);
	bool full = false;
	CHECK_OK(pool->Publish(&full));
	CHECK(full && same_mirror(dev->words, m));
	for (uint32_t id = 0; id < m.TotalPages(); ++id)
		CHECK(m.HasPage(id) ? m.WrittenRange(id) == (hashdag_gb300::PageRange{0, wpp}) : !m.IsDirty(id));
	m.ClearDirty();
	for (int round = 0; round < 4; ++round) {
		const std::vector<uint32_t> before = dev->words.BucketWords();
		append_nodes(dev->words, 500 + 700 * round, 64 + 200 * round);
		CHECK_OK(pool->Publish(&full));
		CHECK(!full && same_mirror(dev->words, m));
		// the written range of every page: the words [old, new) of its bucket on it
		std::vector<hashdag_gb300::PageRange> want(m.TotalPages());
		for (uint32_t b = 0; b < m.TotalBuckets(); ++b)
			for (uint32_t w = before[b]; w < dev->words.BucketWords()[b]; ++w) {
				const uint32_t page = (b << c.page_bits_per_bucket) | (w >> c.word_bits_per_page);
				want[page].unite(w & (wpp - 1u), (w & (wpp - 1u)) + 1u);
			}
		for (uint32_t id = 0; id < m.TotalPages(); ++id)
			CHECK(m.WrittenRange(id) == want[id] && !m.IsFreed(id));
		m.ClearDirty();
	}
	CHECK_OK(pool->Publish(&full)); // nothing new
	CHECK(!full);
	for (uint32_t id = 0; id < m.TotalPages(); ++id)
		CHECK(!m.IsDirty(id));
	// a rewrite (as a collection does): buckets 0..9 emptied, their pages freed,
	// another bucket's words changed in place
	++dev->epoch;
	std::vector<uint32_t> gone;
	for (uint32_t b = 0; b < 10; ++b) {
		for (uint32_t p = 0; p < (1u << c.page_bits_per_bucket); ++p) {
			const uint32_t id = (b << c.page_bits_per_bucket) | p;
			if (dev->words.HasPage(id)) {
				dev->words.FreePage(id);
				gone.push_back(id);
			}
		}
		dev->words.GetBucketRefWords(b) = 0;
	}
	CHECK(!gone.empty());
	const uint32_t w7 = 7u;
	dev->words.WritePage(20u << c.page_bits_per_bucket, 0, std::span<const uint32_t>(&w7, 1));
	CHECK_OK(pool->Publish(&full));
	CHECK(full && same_mirror(dev->words, m));
	for (uint32_t id : gone)
		CHECK(m.IsFreed(id) && !m.HasPage(id));
	for (uint32_t id = 0; id < m.TotalPages(); ++id)
		if (m.HasPage(id))
			CHECK(m.WrittenRange(id) == (hashdag_gb300::PageRange{0, wpp}));
	m.ClearDirty();
	// a count that went down within an epoch is not an append: full read
	dev->words.GetBucketRefWords(30) = dev->words.GetBucketRefWords(30) / 2;
	CHECK_OK(pool->Publish(&full));
	CHECK(full && same_mirror(dev->words, m));
	m.ClearDirty();
	// Upload: the device takes the mirror's words (a new epoch), and the next
	// Publish has nothing to read
	append_nodes(m, 200, 300);
	const uint64_t e0 = dev->epoch;
	CHECK_OK(pool->Upload());
	CHECK(dev->epoch == e0 + 1 && same_mirror(dev->words, m));
	for (uint32_t id = 0; id < m.TotalPages(); ++id)
		CHECK(!m.IsDirty(id));
	CHECK_OK(pool->Publish(&full));
	CHECK(!full);
	for (uint32_t id = 0; id < m.TotalPages(); ++id)
		CHECK(!m.IsDirty(id));
	return 0;
}

static int check_dump(const char *dir) {
	const hd_config c = small_config();
	HostPoolMirror m(c);
	append_nodes(m, 4000, 500);
	const std::string path = std::string(dir) + "/pool.hdmp";
	CHECK(m.Save(path.c_str()));
	HostPoolMirror n(c);
	CHECK(n.Load(path.c_str()) && same_mirror(m, n));
	for (uint32_t id = 0; id < n.TotalPages(); ++id)
		CHECK(n.HasPage(id) ? n.WrittenRange(id) == (hashdag_gb300::PageRange{0, n.WordsPerPage()}) : !n.IsDirty(id));
	hd_config other = c;
	other.bucket_bits_each_level[3] = 9;
	HostPoolMirror o(other);
	CHECK(!o.Load(path.c_str()) && o.PageIds().empty());
	// a truncated file is refused and leaves the mirror empty
	FILE *f = std::fopen(path.c_str(), "rb");
	CHECK(f != nullptr);
	std::vector<char> bytes(1 << 20);
	const size_t len = std::fread(bytes.data(), 1, bytes.size(), f);
	std::fclose(f);
	const std::string cut = std::string(dir) + "/cut.hdmp";
	f = std::fopen(cut.c_str(), "wb");
	CHECK(f != nullptr && std::fwrite(bytes.data(), 1, len / 2, f) == len / 2);
	std::fclose(f);
	HostPoolMirror t(c);
	CHECK(!t.Load(cut.c_str()) && t.PageIds().empty() && t.BucketWords()[0] == 0);
	return 0;
}

// Loads a dump (any configuration) and saves it again.
static int dump_copy(const char *in, const char *out) {
	FILE *f = std::fopen(in, "rb");
	CHECK(f != nullptr);
	hd_config c{};
	char head[8];
	CHECK(std::fread(head, 1, 8, f) == 8 && std::fread(&c, sizeof c, 1, f) == 1);
	std::fclose(f);
	HostPoolMirror m(c);
	CHECK(m.Load(in));
	CHECK(m.Save(out));
	return 0;
}
#endif

#ifndef HD_FAKE_DEVICE
// Applies the descriptors of file `edits` as the application's editor objects
// through the reference's call forms, one per call, and checks the result
// against one batched pass of the descriptors (a fully deduplicated pool gives
// equal DAGs equal pointers).  Saves the pool to `dump`, prints the root.
static int check_editors(const char *edits, const char *dump) {
	using namespace app;
	FILE *f = std::fopen(edits, "rb");
	CHECK(f != nullptr);
	std::vector<hd_edit_desc> e;
	hd_edit_desc x;
	while (std::fread(&x, sizeof x, 1, f) == 1)
		e.push_back(x);
	std::fclose(f);
	CHECK(!e.empty());
	hd_config c{};
	// the configuration follows the edits' file name: EDITS.cfg holds an hd_config
	const std::string cfg_path = std::string(edits) + ".cfg";
	f = std::fopen(cfg_path.c_str(), "rb");
	CHECK(f != nullptr && std::fread(&c, sizeof c, 1, f) == 1);
	std::fclose(f);
	hd_status st = HD_OK;
	auto pool = GpuNodePool::Create(c, 0, 0, &st);
	CHECK_OK(st);
	BusyPool busy;
	uint32_t root = HD_NULL_PTR;
	for (size_t i = 0; i < e.size(); ++i) {
		const hd_edit_desc &d = e[i];
		const u32vec3 p0{d.p0[0], d.p0[1], d.p0[2]}, p1{d.p1[0], d.p1[1], d.p1[2]};
		hd_edit_desc lowered{};
		// every other edit through Edit(root, editor), the rest through ThreadedEdit
		auto apply = [&](const auto &editor) {
			lowered = hashdag_gb300::LowerEditor(editor);
			root = (i & 1u) ? pool->Edit(root, editor) : pool->ThreadedEdit(&busy, root, editor, 5u);
		};
		if (d.shape == HD_SHAPE_SPHERE && d.op == HD_OP_FILL)
			apply(SphereEditor<EditMode::kFill>{p0, d.r2, {}});
		else if (d.shape == HD_SHAPE_SPHERE)
			apply(SphereEditor<EditMode::kDig>{p0, d.r2, {}});
		else if (d.op == HD_OP_FILL)
			apply(AABBEditor{p0, p1, {}});
		else
			apply(BoxEditor<EditMode::kDig>{p0, p1});
		CHECK_OK(pool->LastStatus());
		CHECK(same_desc(lowered, d));
	}
	// a span of editor objects of one type in one batched pass
	std::vector<SphereEditor<EditMode::kDig>> digs;
	for (const hd_edit_desc &d : e)
		if (d.shape == HD_SHAPE_SPHERE && d.op == HD_OP_DIG)
			digs.push_back({{d.p0[0], d.p0[1], d.p0[2]}, d.r2, {}});
	uint32_t batched = HD_NULL_PTR, dug = HD_NULL_PTR, dug_desc = HD_NULL_PTR;
	CHECK_OK(pool->Edit(HD_NULL_PTR, std::span<const hd_edit_desc>(e), &batched));
	CHECK(batched == root);
	if (!digs.empty()) {
		std::vector<hd_edit_desc> dd;
		for (const auto &g : digs)
			dd.push_back(hashdag_gb300::LowerEditor(g));
		CHECK_OK(pool->Edit(root, std::span<const SphereEditor<EditMode::kDig>>(digs), &dug));
		CHECK_OK(pool->Edit(root, std::span<const hd_edit_desc>(dd), &dug_desc));
		CHECK(dug == dug_desc);
	}
	CHECK_OK(pool->Download());
	CHECK(pool->Mirror().Save(dump));
	std::printf("root %u\n", root);
	return 0;
}
#endif

int main(int argc, char **argv) {
	if (argc < 2) {
		std::printf("usage: gpu_pool_check MODE [ARGS]\n");
		return 2;
	}
	const std::string mode = argv[1];
	int rc = 2;
	if (mode == "mirror")
		rc = check_mirror();
	else if (mode == "lowering")
		rc = check_lowering();
#ifndef HD_FAKE_DEVICE
	else if (mode == "nodevice")
		rc = check_nodevice();
	else if (mode == "device")
		rc = check_device();
	else if (mode == "publish")
		rc = check_publish();
	else if (mode == "color")
		rc = check_color();
	else if (mode == "editors" && argc == 4)
		rc = check_editors(argv[2], argv[3]);
#else
	else if (mode == "fake_publish")
		rc = check_fake_publish();
	else if (mode == "dump" && argc == 3)
		rc = check_dump(argv[2]);
	else if (mode == "dump_copy" && argc == 4)
		rc = dump_copy(argv[2], argv[3]);
#endif
	if (rc == 0)
		std::printf("ok %s\n", argv[1]);
	return rc;
}
