// hd_server.cu -- serving loop over several resident scenes.
//
// Threads:
//   * one edit thread per scene: waits for queued edit requests, takes every
//     queued request that admission lets in (arrival order, up to
//     max_pass_edits edits), runs them as ONE batched pass with hd_edit on the
//     scene's stream, publishes the new root and the results;
//   * ray_slots ray threads, each owning one high-priority stream and its
//     device buffers: take the oldest camera request, read its scene's last
//     published root, trace, copy hits/counters back, publish the result.
// A scene's published root only ever names nodes whose pass has completed
// (hd_edit returns after a stream synchronisation), and passes never rewrite
// committed node words, so ray kernels may read a root while later passes of
// the same pool append to its buckets on another stream.
//
// The reference application runs one edit at a time on a worker pool and
// drops edits that arrive meanwhile (src/main.cpp:280-296); frames trace the
// last set root (src/main.cpp:315-321).  Here nothing is dropped: arrivals
// during a pass are merged into the next one.
#include "hd_internal.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>
#include <unordered_set>

using namespace hd;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
	uint64_t id = 0;
	uint32_t kind = HD_REQ_EDIT;
	uint32_t scene = 0;
	std::vector<hd_edit_desc> edits;
	std::vector<hd_camera> cams;
	uint32_t width = 0, height = 0;
	hd_hit *host_out = nullptr;
	double t_submit = 0.0;
};

struct Scene {
	hd_pool *pool = nullptr;
	uint32_t root = kNull;           // last published root (server mutex)
	std::deque<std::unique_ptr<Request>> queue;
	std::condition_variable cv;      // edit thread waits here
	cudaStream_t stream = nullptr;
	std::thread worker;
	hd_edit_desc *staging = nullptr; // pinned concatenation of one pass's edits
	uint32_t staging_cap = 0;
	uint32_t *h_used = nullptr;      // pinned heap counter readback
	uint64_t used_pages = 0, heap_pages = 0;
	double pages_per_edit = 1.0;
	uint64_t passes = 0;
	bool gc_busy = false;        // a collection runs: no ray request of the scene starts (server mutex)
	uint32_t rays_in_flight = 0; // ray requests of the scene on the device (server mutex)
	uint64_t gc_epoch = 0;       // collections so far (server mutex)
};

struct RaySlot {
	cudaStream_t stream = nullptr;
	hd_hit *d_out = nullptr;
	uint64_t out_cap = 0; // hits
	hd_camera *d_cams = nullptr;
	uint32_t cams_cap = 0;
	unsigned long long *d_ctr = nullptr;
	unsigned long long *h_ctr = nullptr; // pinned
	std::thread worker;
};

double percentile(std::vector<double> v, double q) {
	if (v.empty())
		return 0.0;
	std::sort(v.begin(), v.end());
	const double pos = q * double(v.size() - 1);
	const size_t i = (size_t)pos;
	const double f = pos - double(i);
	return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

} // namespace

struct hd_server {
	hd_server_config cfg{};
	int device = 0;
	Clock::time_point t0;
	std::mutex mu;
	std::condition_variable cv_ray, cv_done, cv_gc;
	std::vector<std::unique_ptr<Scene>> scenes;
	std::vector<std::unique_ptr<RaySlot>> slots;
	std::deque<std::unique_ptr<Request>> ray_queue;
	std::unordered_map<uint64_t, hd_request_result> done; // finished, not yet retrieved
	std::unordered_set<uint64_t> pending;                  // submitted, not finished
	uint64_t next_id = 1, outstanding = 0;
	bool stop = false;
	bool paused = false; // no new pass or ray request starts while set
	// statistics
	std::vector<double> lat_edit, lat_cam;
	uint64_t refused = 0, failed = 0, edit_passes = 0, edits_applied = 0, rays_traced = 0, gc_runs = 0;
	uint32_t max_pass_requests = 0;
	double gc_ms = 0.0;

	double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }

	// server mutex held
	void publish(hd_request_result &r) {
		r.t_done_ms = now_ms();
		const double lat = r.t_done_ms - r.t_submit_ms;
		if (r.kind == HD_REQ_EDIT)
			lat_edit.push_back(lat);
		else
			lat_cam.push_back(lat);
		if (!r.admitted)
			++refused;
		else if (r.status != HD_OK)
			++failed;
		done[r.id] = r;
		pending.erase(r.id);
		--outstanding;
	}

	void edit_loop(Scene &sc, uint32_t scene_idx);
	void ray_loop(RaySlot &slot);
	hd_status collect(Scene &sc, std::vector<uint32_t> &roots);
};

namespace {

hd_request_result base_result(const Request &q) {
	hd_request_result r{};
	r.id = q.id;
	r.kind = q.kind;
	r.scene = q.scene;
	r.status = HD_OK;
	r.admitted = 1;
	r.root_in = r.root = kNull;
	r.t_submit_ms = q.t_submit;
	return r;
}

// Heap pages the pool has handed out (physical page 0 is the zero page).
hd_status read_used_pages(Scene &sc) {
	if (cudaMemcpyAsync(sc.h_used, sc.pool->P.counters + kCtrHeapNext, 4, cudaMemcpyDeviceToHost, sc.stream) !=
	        cudaSuccess ||
	    cudaStreamSynchronize(sc.stream) != cudaSuccess)
		return HD_ERR_CUDA;
	sc.used_pages = std::min<uint64_t>(sc.h_used[0], sc.heap_pages) - 1;
	return HD_OK;
}

} // namespace

void hd_server::edit_loop(Scene &sc, uint32_t scene_idx) {
	cudaSetDevice(device);
	const uint64_t reserve = cfg.reserve_pages ? cfg.reserve_pages : std::max<uint64_t>(sc.heap_pages / 64, 1);
	for (;;) {
		std::vector<std::unique_ptr<Request>> take;
		uint32_t root_in;
		uint64_t n_edits = 0;
		{
			std::unique_lock<std::mutex> lk(mu);
			sc.cv.wait(lk, [&] { return stop || (!paused && !sc.queue.empty()); });
			if (sc.queue.empty())
				return; // stop requested and nothing left
			const uint64_t free_pages = sc.heap_pages - 1 - std::min(sc.used_pages, sc.heap_pages - 1);
			const double budget = free_pages > reserve ? double(free_pages - reserve) : 0.0;
			double need = 0.0;
			while (!sc.queue.empty()) {
				Request &q = *sc.queue.front();
				const double est = double(q.edits.size()) * sc.pages_per_edit;
				if (take.empty() && est > budget) { // does not fit even alone: refuse
					hd_request_result r = base_result(q);
					r.status = HD_ERR_POOL_OOM;
					r.admitted = 0;
					r.root_in = r.root = sc.root;
					r.gc_epoch = sc.gc_epoch;
					r.t_start_ms = now_ms();
					publish(r);
					sc.queue.pop_front();
					continue;
				}
				if (!take.empty() && (n_edits + q.edits.size() > cfg.max_pass_edits || need + est > budget))
					break;
				need += est;
				n_edits += q.edits.size();
				take.push_back(std::move(sc.queue.front()));
				sc.queue.pop_front();
			}
			if (take.empty()) {
				cv_done.notify_all();
				continue;
			}
			root_in = sc.root;
		}
		const double t_start = now_ms();
		// concatenate into pinned staging
		if (n_edits > sc.staging_cap) {
			if (sc.staging)
				cudaFreeHost(sc.staging);
			sc.staging = nullptr;
			sc.staging_cap = 0;
			if (cudaMallocHost((void **)&sc.staging, n_edits * sizeof(hd_edit_desc)) == cudaSuccess)
				sc.staging_cap = (uint32_t)n_edits;
		}
		std::vector<hd_request_result> res;
		res.reserve(take.size());
		for (auto &q : take) {
			res.push_back(base_result(*q));
			res.back().t_start_ms = t_start;
			res.back().root_in = root_in;
		}
		uint64_t used_before = sc.used_pages;
		uint32_t root = root_in;
		hd_status st = HD_OK;
		bool gc_held = false; // a collection ran: ray requests of the scene wait until the publish below
		if (!sc.staging) {
			st = HD_ERR_POOL_OOM; // no pinned staging memory: host allocation failed
		} else {
			uint64_t off = 0;
			for (auto &q : take) {
				std::memcpy(sc.staging + off, q->edits.data(), q->edits.size() * sizeof(hd_edit_desc));
				off += q->edits.size();
			}
			st = hd_edit(sc.pool, root_in, sc.staging, (uint32_t)n_edits, &root, sc.stream);
			if (st == HD_ERR_POOL_OOM && cfg.gc_free_fraction > 0.0) {
				// the heap ran out during the pass: collect (the failed pass's words
				// and lost pages go with the garbage) and run the pass once more
				std::vector<uint32_t> keep{root_in};
				if (collect(sc, keep) == HD_OK) {
					root_in = keep[0];
					for (auto &r : res)
						r.root_in = root_in;
					used_before = sc.used_pages;
					root = root_in;
					st = hd_edit(sc.pool, root_in, sc.staging, (uint32_t)n_edits, &root, sc.stream);
				}
				gc_held = true;
			}
		}
		const uint64_t pass_id = ++sc.passes;
		if (st == HD_OK || take.size() == 1) {
			for (size_t i = 0; i < take.size(); ++i) {
				res[i].status = st;
				res[i].root = root;
				res[i].pass_id = pass_id;
				res[i].pass_requests = (uint32_t)take.size();
				res[i].pass_edits = (uint32_t)n_edits;
			}
		} else {
			// the merged pass failed: each request alone, in order, from the same input root
			root = root_in;
			uint64_t off = 0;
			for (size_t i = 0; i < take.size(); ++i) {
				const uint32_t n = (uint32_t)take[i]->edits.size();
				uint32_t r = root;
				const hd_status si = hd_edit(sc.pool, root, sc.staging + off, n, &r, sc.stream);
				off += n;
				if (si == HD_OK)
					root = r;
				res[i].status = si;
				res[i].root = root;
				res[i].pass_id = pass_id;
				res[i].pass_requests = 1;
				res[i].pass_edits = n;
				if (i + 1 < take.size())
					res[i + 1].root_in = root;
			}
		}
		read_used_pages(sc);
		if (n_edits && sc.used_pages >= used_before) {
			const double per = double(sc.used_pages - used_before) / double(n_edits);
			sc.pages_per_edit = sc.passes == 1 ? std::max(per, 1e-3) : 0.75 * sc.pages_per_edit + 0.25 * per;
			sc.pages_per_edit = std::max(sc.pages_per_edit, 1e-3);
		}
		// collect before publishing, so every root a client receives stays
		// valid until the scene's next pass (the pass's input and output roots
		// are kept and remapped)
		const uint64_t free_pages = sc.heap_pages - 1 - std::min(sc.used_pages, sc.heap_pages - 1);
		if (cfg.gc_free_fraction > 0.0 && double(free_pages) < cfg.gc_free_fraction * double(sc.heap_pages)) {
			gc_held = true;
			std::vector<uint32_t> keep;
			keep.reserve(2 * res.size() + 1);
			keep.push_back(root);
			for (auto &r : res) {
				keep.push_back(r.root_in);
				keep.push_back(r.root);
			}
			if (collect(sc, keep) == HD_OK) {
				root = keep[0];
				for (size_t i = 0; i < res.size(); ++i) {
					res[i].root_in = keep[1 + 2 * i];
					res[i].root = keep[2 + 2 * i];
				}
			}
		}
		{
			std::lock_guard<std::mutex> lk(mu);
			sc.root = root;
			sc.gc_busy = false; // ray requests see the remapped root from here on
			++edit_passes;
			max_pass_requests = std::max<uint32_t>(max_pass_requests, (uint32_t)take.size());
			for (size_t i = 0; i < take.size(); ++i) {
				if (res[i].status == HD_OK)
					edits_applied += take[i]->edits.size();
				res[i].gc_epoch = sc.gc_epoch;
				publish(res[i]);
			}
		}
		cv_done.notify_all();
		if (gc_held)
			cv_ray.notify_all();
		(void)scene_idx;
	}
}

// Collects a scene between two of its passes (the edit thread runs this, so
// its queued edits wait and merge into the next pass): waits until none of
// its ray requests is on the device, keeps the nodes `roots` reach and
// remaps them in place.
hd_status hd_server::collect(Scene &sc, std::vector<uint32_t> &roots) {
	{
		std::unique_lock<std::mutex> lk(mu);
		sc.gc_busy = true;
		cv_gc.wait(lk, [&] { return sc.rays_in_flight == 0; });
	}
	const double t0 = now_ms();
	const hd_status st = hd_gc(sc.pool, roots.data(), (uint32_t)roots.size(), nullptr);
	if (st)
		fprintf(stderr, "hashdag_gb300: server collection failed: %s\n", hd_status_string(st));
	cudaSetDevice(device);
	read_used_pages(sc);
	{
		std::lock_guard<std::mutex> lk(mu);
		if (!st)
			++sc.gc_epoch;
		++gc_runs;
		gc_ms += now_ms() - t0;
	}
	return st; // gc_busy stays set until the caller has published the remapped root
}

void hd_server::ray_loop(RaySlot &slot) {
	cudaSetDevice(device);
	for (;;) {
		std::unique_ptr<Request> q;
		uint32_t root;
		hd_pool *pool;
		uint64_t epoch;
		{
			std::unique_lock<std::mutex> lk(mu);
			cv_ray.wait(lk, [&] { return stop || (!paused && !ray_queue.empty()); });
			if (ray_queue.empty())
				return;
			q = std::move(ray_queue.front());
			ray_queue.pop_front();
			Scene &s = *scenes[q->scene];
			cv_ray.wait(lk, [&] { return !s.gc_busy; }); // its pool is being rewritten
			root = s.root; // snapshot: last finished pass
			pool = s.pool;
			epoch = s.gc_epoch;
			++s.rays_in_flight;
		}
		hd_request_result r = base_result(*q);
		r.t_start_ms = now_ms();
		r.root_in = r.root = root;
		const uint32_t nc = (uint32_t)q->cams.size();
		const uint64_t rays = (uint64_t)nc * q->width * q->height;
		r.rays = rays;
		hd_status st = HD_OK;
		if (rays > slot.out_cap) {
			if (slot.d_out)
				cudaFree(slot.d_out);
			slot.d_out = nullptr;
			slot.out_cap = 0;
			if (cudaMalloc(&slot.d_out, rays * sizeof(hd_hit)) == cudaSuccess)
				slot.out_cap = rays;
			else {
				cudaGetLastError();
				st = HD_ERR_POOL_OOM;
			}
		}
		if (!st && nc > slot.cams_cap) {
			if (slot.d_cams)
				cudaFree(slot.d_cams);
			slot.d_cams = nullptr;
			slot.cams_cap = 0;
			if (cudaMalloc(&slot.d_cams, nc * sizeof(hd_camera)) == cudaSuccess)
				slot.cams_cap = nc;
			else {
				cudaGetLastError();
				st = HD_ERR_POOL_OOM;
			}
		}
		if (!st) {
			cudaStream_t s = slot.stream;
			if (cudaMemcpyAsync(slot.d_cams, q->cams.data(), nc * sizeof(hd_camera), cudaMemcpyHostToDevice, s) !=
			        cudaSuccess ||
			    cudaMemsetAsync(slot.d_ctr, 0, 3 * sizeof(unsigned long long), s) != cudaSuccess)
				st = HD_ERR_CUDA;
			if (!st)
				st = hd_launch_pinhole(pool, root, slot.d_cams, nc, q->width, q->height, slot.d_out,
				                       reinterpret_cast<uint64_t *>(slot.d_ctr), s);
			if (!st && q->host_out &&
			    cudaMemcpyAsync(q->host_out, slot.d_out, rays * sizeof(hd_hit), cudaMemcpyDeviceToHost, s) !=
			        cudaSuccess)
				st = HD_ERR_CUDA;
			if (!st && (cudaMemcpyAsync(slot.h_ctr, slot.d_ctr, 3 * sizeof(unsigned long long),
			                            cudaMemcpyDeviceToHost, s) != cudaSuccess ||
			            cudaStreamSynchronize(s) != cudaSuccess))
				st = HD_ERR_CUDA;
			if (!st) {
				r.steps = slot.h_ctr[0];
				r.node_words = slot.h_ctr[1];
				r.hits = slot.h_ctr[2];
			}
		}
		r.status = st;
		r.gc_epoch = epoch;
		{
			std::lock_guard<std::mutex> lk(mu);
			if (!st)
				rays_traced += rays;
			--scenes[r.scene]->rays_in_flight;
			publish(r);
		}
		cv_done.notify_all();
		cv_gc.notify_all();
	}
}

namespace {

void server_free(hd_server *s) {
	if (!s)
		return;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	for (auto &sc : s->scenes)
		sc->cv.notify_all();
	s->cv_ray.notify_all();
	for (auto &sc : s->scenes)
		if (sc->worker.joinable())
			sc->worker.join();
	for (auto &sl : s->slots)
		if (sl->worker.joinable())
			sl->worker.join();
	cudaSetDevice(s->device);
	for (auto &sc : s->scenes) {
		if (sc->stream)
			cudaStreamDestroy(sc->stream);
		if (sc->staging)
			cudaFreeHost(sc->staging);
		if (sc->h_used)
			cudaFreeHost(sc->h_used);
	}
	for (auto &sl : s->slots) {
		if (sl->stream)
			cudaStreamDestroy(sl->stream);
		cudaFree(sl->d_out);
		cudaFree(sl->d_cams);
		cudaFree(sl->d_ctr);
		if (sl->h_ctr)
			cudaFreeHost(sl->h_ctr);
	}
	delete s;
}

} // namespace

extern "C" {

hd_status hd_server_create(hd_pool *const *pools, const uint32_t *roots, uint32_t n_scenes,
                           const hd_server_config *config, hd_server **out_server) {
	if (!out_server)
		return HD_ERR_INVALID_ARG;
	*out_server = nullptr;
	if (!pools || !n_scenes)
		return HD_ERR_INVALID_ARG;
	for (uint32_t i = 0; i < n_scenes; ++i)
		if (!pools[i] || pools[i]->device != pools[0]->device)
			return HD_ERR_INVALID_ARG;
	for (uint32_t i = 0; i < n_scenes; ++i)
		for (uint32_t j = 0; j < i; ++j)
			if (pools[i] == pools[j]) // one edit thread per pool: scenes must not share one
				return HD_ERR_INVALID_ARG;
	hd_server *s = new hd_server();
	if (config)
		s->cfg = *config;
	if (!s->cfg.max_pass_edits)
		s->cfg.max_pass_edits = 16384;
	if (!s->cfg.ray_slots)
		s->cfg.ray_slots = 4;
	if (!s->cfg.max_rays_per_request)
		s->cfg.max_rays_per_request = 1u << 24;
	if (!(s->cfg.pages_per_edit_hint > 0.0))
		s->cfg.pages_per_edit_hint = 1.0;
	s->device = pools[0]->device;
	s->t0 = Clock::now();
	if (cudaSetDevice(s->device) != cudaSuccess) {
		delete s;
		return HD_ERR_CUDA;
	}
	int least = 0, greatest = 0;
	cudaDeviceGetStreamPriorityRange(&least, &greatest);
	hd_status st = HD_OK;
	for (uint32_t i = 0; i < n_scenes && !st; ++i) {
		auto sc = std::make_unique<Scene>();
		sc->pool = pools[i];
		sc->root = roots ? roots[i] : kNull;
		sc->heap_pages = pools[i]->P.heap_pages;
		sc->pages_per_edit = s->cfg.pages_per_edit_hint;
		if (cudaStreamCreateWithPriority(&sc->stream, cudaStreamNonBlocking, least) != cudaSuccess ||
		    cudaMallocHost((void **)&sc->h_used, 64) != cudaSuccess)
			st = HD_ERR_CUDA;
		else
			st = read_used_pages(*sc);
		s->scenes.push_back(std::move(sc));
	}
	for (uint32_t i = 0; i < s->cfg.ray_slots && !st; ++i) {
		auto sl = std::make_unique<RaySlot>();
		if (cudaStreamCreateWithPriority(&sl->stream, cudaStreamNonBlocking, greatest) != cudaSuccess ||
		    cudaMalloc(&sl->d_ctr, 4 * sizeof(unsigned long long)) != cudaSuccess ||
		    cudaMallocHost((void **)&sl->h_ctr, 4 * sizeof(unsigned long long)) != cudaSuccess)
			st = HD_ERR_CUDA;
		s->slots.push_back(std::move(sl));
	}
	if (st) {
		cudaGetLastError();
		server_free(s);
		return st;
	}
	for (uint32_t i = 0; i < n_scenes; ++i) {
		Scene *sc = s->scenes[i].get();
		sc->worker = std::thread([s, sc, i] { s->edit_loop(*sc, i); });
	}
	for (auto &sl : s->slots) {
		RaySlot *p = sl.get();
		p->worker = std::thread([s, p] { s->ray_loop(*p); });
	}
	*out_server = s;
	return HD_OK;
}

void hd_server_destroy(hd_server *server) {
	if (!server)
		return;
	hd_server_pause(server, 0);
	hd_server_drain(server);
	server_free(server);
}

hd_status hd_server_submit_edits(hd_server *server, uint32_t scene, const hd_edit_desc *edits, uint32_t n,
                                 uint64_t *out_id) {
	if (!server || !out_id || scene >= server->scenes.size() || (n && !edits))
		return HD_ERR_INVALID_ARG;
	auto q = std::make_unique<Request>();
	q->kind = HD_REQ_EDIT;
	q->scene = scene;
	q->edits.assign(edits, edits + n);
	Scene &sc = *server->scenes[scene];
	{
		std::lock_guard<std::mutex> lk(server->mu);
		if (server->stop)
			return HD_ERR_INVALID_ARG;
		q->id = server->next_id++;
		q->t_submit = server->now_ms();
		*out_id = q->id;
		++server->outstanding;
		server->pending.insert(q->id);
		if (n == 0) { // nothing to apply: finished at once with the current root
			hd_request_result r = base_result(*q);
			r.root_in = r.root = sc.root;
			r.gc_epoch = sc.gc_epoch;
			r.t_start_ms = q->t_submit;
			server->publish(r);
			server->cv_done.notify_all();
			return HD_OK;
		}
		sc.queue.push_back(std::move(q));
	}
	sc.cv.notify_one();
	return HD_OK;
}

hd_status hd_server_submit_camera(hd_server *server, uint32_t scene, const hd_camera *cameras, uint32_t n_cameras,
                                  uint32_t width, uint32_t height, hd_hit *host_out, uint64_t *out_id) {
	if (!server || !out_id || scene >= server->scenes.size() || !cameras || !n_cameras || !width || !height)
		return HD_ERR_INVALID_ARG;
	const uint64_t rays = (uint64_t)n_cameras * width * height;
	if (rays > server->cfg.max_rays_per_request)
		return HD_ERR_INVALID_ARG;
	auto q = std::make_unique<Request>();
	q->kind = HD_REQ_CAMERA;
	q->scene = scene;
	q->cams.assign(cameras, cameras + n_cameras);
	q->width = width;
	q->height = height;
	q->host_out = host_out;
	{
		std::lock_guard<std::mutex> lk(server->mu);
		if (server->stop)
			return HD_ERR_INVALID_ARG;
		q->id = server->next_id++;
		q->t_submit = server->now_ms();
		*out_id = q->id;
		++server->outstanding;
		server->pending.insert(q->id);
		server->ray_queue.push_back(std::move(q));
	}
	server->cv_ray.notify_one();
	return HD_OK;
}

hd_status hd_server_wait(hd_server *server, uint64_t id, double timeout_ms, hd_request_result *out) {
	if (!server || !out)
		return HD_ERR_INVALID_ARG;
	std::unique_lock<std::mutex> lk(server->mu);
	if (!server->pending.count(id) && !server->done.count(id))
		return HD_ERR_INVALID_ARG; // unknown or already retrieved
	auto ready = [&] { return server->done.count(id) != 0; };
	if (timeout_ms < 0)
		server->cv_done.wait(lk, ready);
	else if (!server->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready))
		return HD_ERR_TIMEOUT;
	auto it = server->done.find(id);
	*out = it->second;
	server->done.erase(it);
	return HD_OK;
}

hd_status hd_server_pause(hd_server *server, int paused) {
	if (!server)
		return HD_ERR_INVALID_ARG;
	{
		std::lock_guard<std::mutex> lk(server->mu);
		server->paused = paused != 0;
	}
	for (auto &sc : server->scenes)
		sc->cv.notify_all();
	server->cv_ray.notify_all();
	return HD_OK;
}

hd_status hd_server_drain(hd_server *server) {
	if (!server)
		return HD_ERR_INVALID_ARG;
	std::unique_lock<std::mutex> lk(server->mu);
	if (server->paused && server->outstanding)
		return HD_ERR_INVALID_ARG; // would never return: nothing starts while paused
	server->cv_done.wait(lk, [&] { return server->outstanding == 0; });
	return HD_OK;
}

hd_status hd_server_scene_root(hd_server *server, uint32_t scene, uint32_t *out_root) {
	if (!server || !out_root || scene >= server->scenes.size())
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(server->mu);
	*out_root = server->scenes[scene]->root;
	return HD_OK;
}

hd_status hd_server_get_stats(hd_server *server, hd_server_stats *out) {
	if (!server || !out)
		return HD_ERR_INVALID_ARG;
	std::lock_guard<std::mutex> lk(server->mu);
	*out = hd_server_stats{};
	out->edit_requests = server->lat_edit.size();
	out->camera_requests = server->lat_cam.size();
	out->refused = server->refused;
	out->failed = server->failed;
	out->edit_passes = server->edit_passes;
	out->edits_applied = server->edits_applied;
	out->rays_traced = server->rays_traced;
	out->max_pass_requests = server->max_pass_requests;
	out->queued = (uint32_t)std::min<uint64_t>(server->outstanding, 0xFFFFFFFFu);
	out->edit_p50_ms = percentile(server->lat_edit, 0.50);
	out->edit_p99_ms = percentile(server->lat_edit, 0.99);
	out->camera_p50_ms = percentile(server->lat_cam, 0.50);
	out->camera_p99_ms = percentile(server->lat_cam, 0.99);
	out->gc_runs = server->gc_runs;
	out->gc_ms = server->gc_ms;
	return HD_OK;
}

} // extern "C"
