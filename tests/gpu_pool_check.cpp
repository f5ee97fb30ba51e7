// gpu_pool_check.cpp -- checks of the C++ host side of the pool
// (include/hashdag_gpu_pool.hpp, include/hashdag_host_mirror.hpp), linked
// against libhashdag_gb300.so by tests/test_cpp_pool.py.
//
//   gpu_pool_check mirror    HostPoolMirror's storage hooks on their own
//   gpu_pool_check nodevice  GpuNodePool::Create with no usable device:
//                            nullptr and HD_ERR_NO_DEVICE, like DAGNodePool::Create
//   gpu_pool_check device    on a GPU: edits on the device, Download into the
//                            mirror, Upload of that mirror into a second pool
//                            (word for word the same pool, same filled
//                            pointers), the same further edits on both, and
//                            occupancy against the edits' own predicates;
//                            then GC through the class and the same check.
// Prints "ok <mode>" and exits 0, or prints the first failure and exits 1.
#include "hashdag_gpu_pool.hpp"

#include <cstdio>
#include <cstring>
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

static hd_config small_config() {
	hd_config c;
	// DefaultConfig for a 256^3 grid: level_count 8, 9 top levels of 2^10
	// buckets (so every one of the 7 node levels), 512-word pages, 4 per bucket
	hd_config_default(8, 9, 9, 2, 10, 16, &c);
	return c;
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

static bool same_mirror(const HostPoolMirror &a, const HostPoolMirror &b) {
	if (a.BucketWords() != b.BucketWords() || a.PageIds() != b.PageIds())
		return false;
	for (uint32_t id : a.PageIds())
		if (std::memcmp(a.ReadPage(id), b.ReadPage(id), a.WordsPerPage() * 4u) != 0)
			return false;
	return true;
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

int main(int argc, char **argv) {
	if (argc != 2) {
		std::printf("usage: gpu_pool_check mirror|nodevice|device\n");
		return 2;
	}
	int rc = 2;
	if (!std::strcmp(argv[1], "mirror"))
		rc = check_mirror();
	else if (!std::strcmp(argv[1], "nodevice"))
		rc = check_nodevice();
	else if (!std::strcmp(argv[1], "device"))
		rc = check_device();
	if (rc == 0)
		std::printf("ok %s\n", argv[1]);
	return rc;
}
