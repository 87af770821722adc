// Continuous-batching request loop over the propagation plans (host code only).
//
// The reference's backend is one blocking call per sample (bpm_backend.cpp:7-164). Here a
// server thread keeps several samples ("requests") in flight on one GPU:
//   * submit() parses and validates a request in the caller's thread (the reference's
//     messages and error codes), estimates its device memory and queues it;
//   * admission is first-come first-served under a device-memory budget: the head of the
//     queue is admitted when its estimate fits next to the requests in flight, its director
//     is uploaded and its entrance operators recorded;
//   * every scheduling round advances each request in flight by as many slabs as fit a
//     voxel-step quantum (at least one) on its own CUDA streams, so requests of different
//     meshes run side by side, small ones finish in few rounds, and new ones join at slab
//     boundaries as earlier ones finish and free their memory;
//   * a finished request gets its exit operators, screen filter and the copy into the
//     caller's buffer; its memory returns to the budget.
// Each request runs exactly the launch sequence of a standalone run of the same plan, so its
// results do not depend on what else is in flight.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/nbpm.h"
#include "host_settings.h"
#include "plan_iface.h"

namespace nbpm {
namespace {

double now_s() {
	using namespace std::chrono;
	return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
	long long id = 0;
	std::unique_ptr<PlanBase> plan;
	int state = NBPM_REQ_QUEUED;
	int error_code = 0;
	std::string error;
	long long bytes = 0;
	long long vs = 0;
	double t_submit = 0, t_admit = 0, t_done = 0;
	bool cancel = false;
	bool finishing = false;
	int slabs_per_round = 1;
};

}  // namespace

struct Server {
	nbpm_server_options opt;
	std::mutex mu;
	std::condition_variable cv_work, cv_done;
	std::deque<Request*> queue;
	std::vector<Request*> active;
	std::unordered_map<long long, std::unique_ptr<Request>> reqs;
	long long next_id = 1;
	long long used = 0, peak = 0, budget = 0;
	long long n_done = 0, n_failed = 0, n_cancelled = 0, vs_done = 0;
	int rounds = 0;
	bool stop = false;
	std::thread th;

	explicit Server(const nbpm_server_options& o) : opt(o) {
		budget = (long long)(o.hbm_budget_gb * 1e9);
		th = std::thread([this] { loop(); });
	}

	~Server() {
		{
			std::lock_guard<std::mutex> lk(mu);
			stop = true;
			for(Request* r : queue) {
				r->state = NBPM_REQ_CANCELLED;
				r->plan.reset();
				n_cancelled++;
			}
			queue.clear();
		}
		cv_work.notify_all();
		if(th.joinable()) th.join();
	}

	// Caller holds mu.
	void finish_req(Request* r, int state, int code, const std::string& msg) {
		r->state = state;
		r->error_code = code;
		r->error = msg;
		r->t_done = now_s();
		if(state == NBPM_REQ_DONE) { n_done++; vs_done += r->vs; }
		else if(state == NBPM_REQ_FAILED) n_failed++;
		else n_cancelled++;
		cv_done.notify_all();
	}

	void loop() {
		bool dev_ok = cudaSetDevice(opt.device) == cudaSuccess;
		for(;;) {
			std::vector<Request*> admit;
			{
				std::unique_lock<std::mutex> lk(mu);
				cv_work.wait(lk, [&] { return stop || !queue.empty() || !active.empty(); });
				if(stop && queue.empty() && active.empty()) break;
				// FCFS admission under the memory budget
				while(!queue.empty()) {
					Request* r = queue.front();
					if(r->cancel) {
						queue.pop_front();
						r->plan.reset();
						finish_req(r, NBPM_REQ_CANCELLED, 0, "cancelled");
						continue;
					}
					if(opt.max_active > 0 && (int)(active.size() + admit.size()) >= opt.max_active) break;
					if(used + r->bytes > budget) break;
					queue.pop_front();
					used += r->bytes;
					peak = std::max(peak, used);
					admit.push_back(r);
				}
			}
			for(Request* r : admit) {
				int code = 0;
				std::string msg;
				try {
					if(!dev_ok) throw BackendError(E_CUDA, "cannot select the server's CUDA device");
					r->plan->setup_device();
					r->plan->upload();
					r->plan->step_begin();
				}
				catch(BackendError& e) { code = e.code; msg = e.what(); }
				catch(std::bad_alloc&) { code = E_MEMORY; msg = "host out of memory"; }
				catch(std::exception& e) { code = E_INTERNAL; msg = e.what(); }
				std::lock_guard<std::mutex> lk(mu);
				r->t_admit = now_s();
				if(code) {
					r->plan.reset();
					used -= r->bytes;
					finish_req(r, NBPM_REQ_FAILED, code, msg);
				}
				else {
					r->state = NBPM_REQ_RUNNING;
					active.push_back(r);
				}
			}
			// one scheduling round: every request in flight advances K slabs
			std::vector<Request*> cur;
			{
				std::lock_guard<std::mutex> lk(mu);
				cur = active;
			}
			std::vector<std::pair<Request*, std::pair<int, std::string>>> failed;
			for(Request* r : cur) {
				try {
					if(!r->finishing) {
						int left = r->plan->step_advance(r->slabs_per_round);
						if(left == 0) {
							r->plan->step_finish();
							r->finishing = true;
						}
					}
				}
				catch(BackendError& e) { failed.push_back({r, {e.code, e.what()}}); }
				catch(std::exception& e) { failed.push_back({r, {E_INTERNAL, e.what()}}); }
			}
			// wait for the round; completed requests leave
			std::vector<Request*> done;
			for(Request* r : cur) {
				bool bad = false;
				for(auto& f : failed) bad |= f.first == r;
				if(bad) continue;
				try {
					r->plan->sync();
					if(r->finishing && r->plan->step_done()) {
						r->plan->host_finish();
						done.push_back(r);
					}
				}
				catch(BackendError& e) { failed.push_back({r, {e.code, e.what()}}); }
			}
			std::lock_guard<std::mutex> lk(mu);
			rounds++;
			for(Request* r : done) {
				r->plan.reset();
				used -= r->bytes;
				active.erase(std::find(active.begin(), active.end(), r));
				finish_req(r, NBPM_REQ_DONE, 0, "");
			}
			for(auto& f : failed) {
				Request* r = f.first;
				r->plan.reset();
				used -= r->bytes;
				active.erase(std::find(active.begin(), active.end(), r));
				finish_req(r, NBPM_REQ_FAILED, f.second.first, f.second.second);
			}
			// cancellation of requests in flight takes effect at the round boundary
			for(size_t i = 0; i < active.size();) {
				Request* r = active[i];
				if(r->cancel) {
					r->plan.reset();
					used -= r->bytes;
					active.erase(active.begin() + i);
					finish_req(r, NBPM_REQ_CANCELLED, 0, "cancelled");
				}
				else i++;
			}
		}
	}

	void info(const Request* r, nbpm_request_info* o) const {
		std::memset(o, 0, sizeof(*o));
		o->state = r->state;
		o->error_code = r->error_code;
		std::snprintf(o->error, sizeof(o->error), "%s", r->error.c_str());
		o->voxel_steps = r->vs;
		o->device_bytes = r->bytes;
		o->queue_ms = r->t_admit > 0 ? 1e3 * (r->t_admit - r->t_submit) : 0;
		o->latency_ms = r->t_done > 0 ? 1e3 * (r->t_done - r->t_submit) : 0;
	}
};

}  // namespace nbpm

using namespace nbpm;

struct nbpm_server {
	std::unique_ptr<Server> s;
};

#define SRV_GUARD(...)                                                                    \
	try { __VA_ARGS__ }                                                                   \
	catch(BackendError& e) { set_last_error(e.what()); return e.code; }                   \
	catch(std::bad_alloc&) { set_last_error("host out of memory"); return NBPM_ERR_MEMORY; } \
	catch(std::exception& e) { set_last_error(e.what()); return NBPM_ERR_INTERNAL; }      \
	catch(...) { set_last_error("unknown exception"); return NBPM_ERR_INTERNAL; }

extern "C" {

void nbpm_default_server_options(nbpm_server_options* o) {
	if(!o) return;
	std::memset(o, 0, sizeof(*o));
	o->precision = NBPM_FP32;
	o->device = 0;
	o->hbm_budget_gb = 150.0;
	o->slabs_per_round = 8;
	o->max_active = 0;
	o->round_voxel_steps = 4e8;
}

int nbpm_server_create(const nbpm_server_options* opts, nbpm_server** out) {
	SRV_GUARD({
		if(!out) { set_last_error("null argument"); return NBPM_ERR_ARG; }
		*out = nullptr;
		nbpm_server_options o;
		nbpm_default_server_options(&o);
		if(opts) o = *opts;
		if(o.precision != NBPM_FP32 && o.precision != NBPM_FP64) { set_last_error("unknown precision"); return NBPM_ERR_ARG; }
		if(!(o.hbm_budget_gb > 0)) { set_last_error("hbm_budget_gb must be > 0"); return NBPM_ERR_ARG; }
		std::unique_ptr<nbpm_server> h(new nbpm_server());
		h->s.reset(new Server(o));
		*out = h.release();
		return 0;
	})
}

int nbpm_server_destroy(nbpm_server* h) {
	delete h;
	return 0;
}

int nbpm_server_submit(nbpm_server* h, const nbpm_sample* req, long long* id) {
	SRV_GUARD({
		if(!h || !req || !id) { set_last_error("null argument"); return NBPM_ERR_ARG; }
		Server& S = *h->s;
		nbpm_options po;
		nbpm_default_options(&po);
		po.precision = S.opt.precision;
		po.device = S.opt.device;
		po.groups_per_pass = 0;
		po.use_graph = 0;
		std::unique_ptr<Request> r(new Request());
		r->plan = make_plan_host(1, req, po);
		r->bytes = r->plan->estimate_bytes();
		r->vs = r->plan->voxel_steps();
		{
			int nslab = std::max(1, r->plan->slabs());
			double per_slab = (double)r->vs / nslab;
			r->slabs_per_round = S.opt.round_voxel_steps > 0
				? (int)std::max(1.0, std::min((double)nslab, std::floor(S.opt.round_voxel_steps / std::max(1.0, per_slab))))
				: std::max(1, S.opt.slabs_per_round);
		}
		if(r->bytes > S.budget) {
			char msg[200];
			std::snprintf(msg, sizeof msg, "request needs %.3f GB of device memory, above the server budget of %.3f GB",
				r->bytes / 1e9, S.budget / 1e9);
			set_last_error(msg);
			return NBPM_ERR_MEMORY;
		}
		r->t_submit = now_s();
		{
			std::lock_guard<std::mutex> lk(S.mu);
			if(S.stop) { set_last_error("server is shutting down"); return NBPM_ERR_ARG; }
			r->id = S.next_id++;
			*id = r->id;
			S.queue.push_back(r.get());
			S.reqs[r->id] = std::move(r);
		}
		S.cv_work.notify_all();
		return 0;
	})
}

int nbpm_server_poll(nbpm_server* h, long long id, nbpm_request_info* info) {
	if(!h || !info) { set_last_error("null argument"); return NBPM_ERR_ARG; }
	Server& S = *h->s;
	std::lock_guard<std::mutex> lk(S.mu);
	auto it = S.reqs.find(id);
	if(it == S.reqs.end()) { set_last_error("unknown request id"); return NBPM_ERR_ARG; }
	S.info(it->second.get(), info);
	return 0;
}

int nbpm_server_wait(nbpm_server* h, long long id, double timeout_s, nbpm_request_info* info) {
	if(!h) { set_last_error("null argument"); return NBPM_ERR_ARG; }
	Server& S = *h->s;
	std::unique_lock<std::mutex> lk(S.mu);
	auto it = S.reqs.find(id);
	if(it == S.reqs.end()) { set_last_error("unknown request id"); return NBPM_ERR_ARG; }
	Request* r = it->second.get();
	auto finished = [&] { return r->state >= NBPM_REQ_DONE; };
	if(timeout_s < 0) S.cv_done.wait(lk, finished);
	else if(!S.cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished)) {
		if(info) S.info(r, info);
		set_last_error("timed out");
		return NBPM_ERR_TIMEOUT;
	}
	if(info) S.info(r, info);
	return 0;
}

int nbpm_server_cancel(nbpm_server* h, long long id) {
	if(!h) { set_last_error("null argument"); return NBPM_ERR_ARG; }
	Server& S = *h->s;
	{
		std::lock_guard<std::mutex> lk(S.mu);
		auto it = S.reqs.find(id);
		if(it == S.reqs.end()) { set_last_error("unknown request id"); return NBPM_ERR_ARG; }
		it->second->cancel = true;
	}
	S.cv_work.notify_all();
	return 0;
}

int nbpm_server_release(nbpm_server* h, long long id) {
	if(!h) { set_last_error("null argument"); return NBPM_ERR_ARG; }
	Server& S = *h->s;
	std::lock_guard<std::mutex> lk(S.mu);
	auto it = S.reqs.find(id);
	if(it == S.reqs.end()) { set_last_error("unknown request id"); return NBPM_ERR_ARG; }
	if(it->second->state < NBPM_REQ_DONE) { set_last_error("request still queued or running"); return NBPM_ERR_ARG; }
	S.reqs.erase(it);
	return 0;
}

int nbpm_server_get_stats(nbpm_server* h, nbpm_server_stats* st) {
	if(!h || !st) { set_last_error("null argument"); return NBPM_ERR_ARG; }
	Server& S = *h->s;
	std::lock_guard<std::mutex> lk(S.mu);
	std::memset(st, 0, sizeof(*st));
	st->queued = (int)S.queue.size();
	st->running = (int)S.active.size();
	st->done = S.n_done;
	st->failed = S.n_failed;
	st->cancelled = S.n_cancelled;
	st->bytes_in_use = S.used;
	st->peak_bytes = S.peak;
	st->budget_bytes = S.budget;
	st->voxel_steps_done = S.vs_done;
	st->rounds = S.rounds;
	return 0;
}

}  // extern "C"
