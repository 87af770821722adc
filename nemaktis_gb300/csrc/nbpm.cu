// libnbpm: host orchestration and C ABI of the GB300 bpm backend.
//
// Replaces the reference's backend entry (BeamPropagationSolver/src/PythonBackend/
// bpm_backend.cpp:7-164) and the orchestration of BPMIteration::propagate_fields
// (BeamPropagationLib/BPMIteration.cpp:53-177) + ScreenOutput::apply_no_export
// (PostprocessorLib/ScreenOutput.cpp:184-224). All arithmetic runs in the kernels of
// bpm_kernels.cuh and fft_kernels.cuh; the host parses, validates, allocates, uploads and
// launches (inside one captured CUDA graph per plan).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <stdexcept>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/nbpm.h"
#include "bpm_kernels.cuh"
#include "fft_kernels.cuh"
#include "plan_iface.h"
#include "vti_writer.h"
#include "host_settings.h"
#include "solve_dispatch.cuh"
#include "solve_config.h"

namespace nbpm {

static thread_local std::string g_last_error;

// Shared with the other translation units of the library.
void set_last_error(const std::string& m) { g_last_error = m; }

// Tuned line-solve configurations, per shape key (direction | precision | mesh | slots per
// wavelength | wavelengths per pass | Woodbury steps | SMs), shared by every plan of the process.
// With NBPM_TUNE_CACHE set to a file name, entries are read from that file when the cache is
// first used and each new entry is appended to it, so later processes skip the timing runs.
namespace {
struct TuneCache {
	std::mutex m;
	std::map<std::string, std::string> entries;
	bool loaded = false;
	std::string file;
};
TuneCache& tune_cache() {
	static TuneCache* c = new TuneCache();  // never destroyed (see plan_cache)
	return *c;
}
void tune_cache_load(TuneCache& c) {
	if(c.loaded) return;
	c.loaded = true;
	const char* f = std::getenv("NBPM_TUNE_CACHE");
	if(!f || !*f) return;
	c.file = f;
	if(FILE* fp = std::fopen(f, "r")) {
		char line[512];
		while(std::fgets(line, sizeof line, fp)) {
			std::string l(line);
			while(!l.empty() && (l.back() == '\n' || l.back() == '\r')) l.pop_back();
			size_t t = l.find('\t');
			if(t != std::string::npos) c.entries[l.substr(0, t)] = l.substr(t + 1);
		}
		std::fclose(fp);
	}
}
}  // namespace

bool tune_cache_get(const std::string& key, std::string& val) {
	TuneCache& c = tune_cache();
	std::lock_guard<std::mutex> lk(c.m);
	tune_cache_load(c);
	auto it = c.entries.find(key);
	if(it == c.entries.end()) return false;
	val = it->second;
	return true;
}

void tune_cache_put(const std::string& key, const std::string& val) {
	TuneCache& c = tune_cache();
	std::lock_guard<std::mutex> lk(c.m);
	tune_cache_load(c);
	c.entries[key] = val;
	if(!c.file.empty())
		if(FILE* fp = std::fopen(c.file.c_str(), "a")) {
			std::fprintf(fp, "%s\t%s\n", key.c_str(), val.c_str());
			std::fclose(fp);
		}
}

void tune_cache_clear() {
	TuneCache& c = tune_cache();
	std::lock_guard<std::mutex> lk(c.m);
	c.entries.clear();
}

#define CK(call)                                                                                   \
	do {                                                                                           \
		cudaError_t e_ = (call);                                                                   \
		if(e_ != cudaSuccess) {                                                                    \
			if(e_ == cudaErrorMemoryAllocation)                                                    \
				throw BackendError(E_MEMORY, std::string("CUDA out of memory: ") + #call);         \
			throw BackendError(E_CUDA, std::string(cudaGetErrorString(e_)) + " at " + #call);      \
		}                                                                                          \
	} while(0)

// ---------------------------------------------------------------------------------------
// Device memory owner.
// ---------------------------------------------------------------------------------------
struct DevBuf {
	void* p = nullptr;
	size_t bytes = 0;
	DevBuf() = default;
	DevBuf(const DevBuf&) = delete;
	DevBuf& operator=(const DevBuf&) = delete;
	~DevBuf() { if(p) cudaFree(p); }
	void alloc(size_t b) {
		if(p) { cudaFree(p); p = nullptr; }
		bytes = b;
		if(b) CK(cudaMalloc(&p, b));
	}
	template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

struct SampleHost {
	BackendSettings s;
	const double* lc = nullptr;
	int fd = 3;
	std::vector<unsigned char> mask;
	std::vector<double> wts;
	bool has_mask = false, has_wts = false;
	double* E = nullptr;  // user buffer, complex128 interleaved
	int G = 0, Nq = 0, spg = 0, slots = 0;
	Geom geom;
	size_t nvox = 0;
	std::vector<GroupParams> gps;
	std::vector<ShiftParams> shifts;
	bool any_shift = false, any_zero_q = false;
	int index = 0;
	ScreenParams sp;
	// bulk output (fields of every plane): [slot][re, im][iz * N + p][Ex, Ey, 0]
	bool bulk = false;
	std::vector<double> bulk_data;
	cx<double>* hstage = nullptr;  // pinned host staging of one pass's plane
	// device
	DevBuf dir, dmask, dwts, F, E0, gpsd, shiftd, partial, wl, nout, qv, bstage;
	// The sample's lane: its own streams (sample 0 uses the plan's), events and workspace, so that
	// the samples of a batch run side by side on the device, each in its own branch of the graph.
	struct Lane {
		cudaStream_t main = nullptr, setup = nullptr;
		bool owns_streams = false;
		cudaEvent_t eFork = nullptr, eJoin = nullptr, eCoef = nullptr, eFac = nullptr, eTrans = nullptr;
		cudaEvent_t eAdi[2] = {nullptr, nullptr};
		cudaEvent_t eNref = nullptr, eNrefFork = nullptr, eEnd = nullptr;
		// workspace: field-sized iterates T, T2 (T3 for the scratch-chunk y solve), eps and
		// coefficient rings, diagonal stencils, double-buffered factor planes / line scalars
		// (slab iz uses half iz & 1), screen and widening buffers
		DevBuf T, T2, T3, Qring, coef, diag, facx, facy, lscx, lscy, scr, stage;
		// transposed-frame y solves: transposed coefficient ring (two slabs) and diagonal stencils
		DevBuf coefT, diagT;
		size_t facx_half = 0, facy_half = 0, lsc_half = 0;
		std::vector<cudaEvent_t*> events() {
			return {&eFork, &eJoin, &eCoef, &eFac, &eTrans, &eAdi[0], &eAdi[1], &eNref, &eNrefFork, &eEnd};
		}
		~Lane() {
			if(main) cudaStreamSynchronize(main);
			if(setup) cudaStreamSynchronize(setup);
			for(cudaEvent_t* e : events()) if(*e) cudaEventDestroy(*e);
			if(owns_streams) {
				if(setup) cudaStreamDestroy(setup);
				if(main) cudaStreamDestroy(main);
			}
		}
	} lane;
	~SampleHost() { if(hstage) cudaFreeHost(hstage); }
};

// One recorded bulk-output copy: the host function scatters the staged plane into the
// sample's bulk arrays.
struct BulkRec {
	SampleHost* h;
	int slot0, nsl, iz;
};

static void CUDART_CB bulk_host_fn(void* p) {
	const BulkRec& r = *static_cast<const BulkRec*>(p);
	SampleHost& h = *r.h;
	const size_t N = (size_t)h.geom.N, Nz = (size_t)h.geom.Nz;
	for(int s = 0; s < r.nsl; s++) {
		size_t slot = (size_t)r.slot0 + s;
		double* re = h.bulk_data.data() + slot * 2 * 3 * N * Nz;
		double* im = re + 3 * N * Nz;
		for(int c = 0; c < 2; c++) {
			const cx<double>* src = h.hstage + ((size_t)s * 2 + c) * N;
			for(size_t p = 0; p < N; p++) {
				size_t o = 3 * ((size_t)r.iz * N + p);
				re[o + c] = src[p].x;
				im[o + c] = src[p].y;
			}
		}
	}
}

// Nearest-index divisions used by the shift operator are computed on the device from nref;
// this kernel restates the SimpleShiftOperator constructor (SimpleShiftOperator.cpp:3-50).
__global__ void k_nref_final(int ngroups, int nblocks, size_t nvox, const double* __restrict__ partial,
		GroupParams* gps) {
	int g = blockIdx.x * blockDim.x + threadIdx.x;
	if(g >= ngroups) return;
	double s = 0;
	for(int b = 0; b < nblocks; b++) s += partial[(size_t)g * nblocks + b];
	gps[g].nref = s / (double)nvox;
}

__global__ void k_shift_params(int ngroups, int Nq, int Nx, int Ny, const GroupParams* __restrict__ gps,
		const double* __restrict__ qv, ShiftParams* sp) {
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if(t >= ngroups * Nq) return;
	int g = t / Nq, q = t % Nq;
	double qx = qv[2 * q], qy = qv[2 * q + 1];
	ShiftParams P;
	P.active = !(qx == 0 && qy == 0);
	double nref = gps[g].nref, dZ = gps[g].dZ, dX = gps[g].dX;
	double arg = -dZ * (qx * qx + qy * qy) / (4 * nref);  // exp(-i*dZ*|q|^2/(4 nref))
	double s, c;
	sincos(arg, &s, &c);
	P.ph_re = c; P.ph_im = s;
	P.msx = P.msy = 0;
	for(int k = 0; k < 4; k++) { P.wx[k] = 0; P.wy[k] = 0; }
	P.wx[1] = P.wy[1] = 1;
	if(Nx > 3) {
		double xs = -dZ * qx / (2 * nref * dX);
		double ms = floor(xs), nu = xs - ms;
		P.msx = (int)ms;
		P.wx[0] = -nu * (1 - nu) * (1 - nu) / 2;
		P.wx[1] = (1 - nu) * (1 + nu - 3 * nu * nu / 2);
		P.wx[2] = nu * (1 + 4 * nu - 3 * nu * nu) / 2;
		P.wx[3] = -nu * nu * (1 - nu) / 2;
	}
	if(Ny > 3) {
		double ys = -dZ * qy / (2 * nref * dX);  // the reference divides by the x spacing
		double ms = floor(ys), nu = ys - ms;
		P.msy = (int)ms;
		P.wy[0] = -nu * (1 - nu) * (1 - nu) / 2;
		P.wy[1] = (1 - nu) * (1 + nu - 3 * nu * nu / 2);
		P.wy[2] = nu * (1 + 4 * nu - 3 * nu * nu) / 2;
		P.wy[3] = -nu * nu * (1 - nu) / 2;
	}
	for(int k = 0; k < 4; k++) { P.fwx[k] = (float)P.wx[k]; P.fwy[k] = (float)P.wy[k]; }
	P.fph_re = (float)P.ph_re; P.fph_im = (float)P.ph_im;
	sp[t] = P;
}

// ---------------------------------------------------------------------------------------
// Plan
// ---------------------------------------------------------------------------------------
template <typename R>
struct Plan : PlanBase {
	nbpm_options opt;
	std::vector<std::unique_ptr<SampleHost>> S;
	// The plan's own streams (sample 0's lane) and, while a sample is recorded, that sample's
	// lane (select()): stream = right-hand-side work and copies, streamB = per-slab setup (eps
	// planes, coefficients, factorisations).
	cudaStream_t stream0 = nullptr, streamB0 = nullptr;
	cudaStream_t stream = nullptr;
	cudaStream_t streamB = nullptr;
	cudaStream_t cs = nullptr;       // stream the next launch goes to
	cudaEvent_t eFork = nullptr, eJoin = nullptr, eCoef = nullptr, eFac = nullptr, eTrans = nullptr, eAdi[2] = {nullptr, nullptr};
	cudaEvent_t eNref = nullptr, eNrefFork = nullptr;
	cudaEvent_t eBatch = nullptr;    // start of a batch recording on the plan's stream
	SampleHost::Lane* W = nullptr;   // workspace of the sample being recorded
	cx<R>* fx_cur = nullptr;
	const cx<R>* ct_cur = nullptr;   // transposed coefficients of the slab being recorded
	cx<R>* fy_cur = nullptr;
	cx<double>* lx_cur = nullptr;
	cx<double>* ly_cur = nullptr;
	cudaGraphExec_t gexec = nullptr;
	cudaEvent_t ev[6];
	std::vector<DevBuf*> tw_bufs;
	std::vector<std::unique_ptr<DevBuf>> tw_store;
	std::vector<std::pair<int, cx<R>*>> tw_tables;
	int launches = 0;
	long long dev_bytes = 0;
	// Live per-kernel timing (nbpm_plan_profile): events around every launch of an eager run.
	struct ProfRec { const char* name; double bytes; cudaEvent_t a, b; };
	bool profiling = false;
	std::vector<ProfRec> prof;
	std::vector<cudaEvent_t> evpool;
	size_t evnext = 0;
	cudaEvent_t pool_event() {
		if(evnext == evpool.size()) {
			cudaEvent_t e;
			CK(cudaEventCreate(&e));
			evpool.push_back(e);
		}
		return evpool[evnext++];
	}
	template <typename F>
	void launch(const char* name, double bytes, F&& fn) {
		if(profiling) {
			// each kernel alone on the device: the launches before it (on either stream) have
			// finished, so the events time this kernel without the overlap of the two streams
			CK(cudaDeviceSynchronize());
			ProfRec r{name, bytes, pool_event(), pool_event()};
			CK(cudaEventRecord(r.a, cs));
			fn();
			CK(cudaEventRecord(r.b, cs));
			prof.push_back(r);
		}
		else fn();
		CK(cudaGetLastError());
		launches++;
	}
	double last_slab_ms = 0;
	size_t smem_limit = 0;
	int nsm = 152;  // streaming multiprocessors of the device (queried at setup)
	// Line-solve configuration per sample (solve_config.h): forced by opts.solve_config, timed
	// per shape by tune() (opts.tune), or the rule-based default.
	std::vector<std::string> tune_notes;  // per sample: how its configuration was chosen
	std::vector<SolveCfg> scfg;

	// Makes h's lane current: its streams, events and workspace.
	void select(SampleHost& h) {
		auto& L = h.lane;
		stream = L.main; streamB = L.setup; cs = stream;
		eFork = L.eFork; eJoin = L.eJoin; eCoef = L.eCoef; eFac = L.eFac; eTrans = L.eTrans;
		eAdi[0] = L.eAdi[0]; eAdi[1] = L.eAdi[1]; eNref = L.eNref; eNrefFork = L.eNrefFork;
		W = &L;
	}

	Plan(const nbpm_options& o) : opt(o) {
		for(auto& e : ev) e = nullptr;
	}
	~Plan() override {
		if(stream0) cudaStreamSynchronize(stream0);
		if(streamB0) cudaStreamSynchronize(streamB0);
		S.clear();  // lanes: their streams and events
		if(eDone) cudaEventDestroy(eDone);
		if(eBatch) cudaEventDestroy(eBatch);
		for(auto e : evpool) cudaEventDestroy(e);
		if(gexec) cudaGraphExecDestroy(gexec);
		for(auto& e : ev) if(e) cudaEventDestroy(e);
		if(streamB0) cudaStreamDestroy(streamB0);
		if(stream0) cudaStreamDestroy(stream0);
	}

	cx<R>* twiddles(int n) {
		for(auto& t : tw_tables) if(t.first == n) return t.second;
		std::vector<cx<R>> h(n);
		const double PI_REF = 3.1415926535897932;
		for(int k = 0; k < n; k++) {
			double a = 2 * PI_REF * (double)k / (double)n;
			h[k] = mk<R>((R)std::cos(a), (R)(-std::sin(a)));
		}
		tw_store.emplace_back(new DevBuf());
		tw_store.back()->alloc(sizeof(cx<R>) * n);
		CK(cudaMemcpy(tw_store.back()->p, h.data(), sizeof(cx<R>) * n, cudaMemcpyHostToDevice));
		dev_bytes += sizeof(cx<R>) * n;
		tw_tables.emplace_back(n, tw_store.back()->as<cx<R>>());
		return tw_tables.back().second;
	}

	void setup_host(int ns, const nbpm_sample* samples) {
		for(int i = 0; i < ns; i++) {
			const nbpm_sample& in = samples[i];
			if(!in.json_str || !in.lc_field_vals || !in.E_field_vals)
				throw BackendError(E_ARG, "null pointer argument");
			std::unique_ptr<SampleHost> h(new SampleHost());
			h->s = parse_settings(in.json_str);
			auto& s = h->s;
			size_t nv = (size_t)s.Nx * s.Ny * s.Nz;
			h->nvox = nv;
			// VectorField(mesh, vals, n) (VectorField.cpp:27-40 / :43-58)
			if(in.n_lc_vals < 0 || nv == 0) throw BackendError(E_SIZE, "Wrong dimension for the user pointer array (VectorField)");
			int fd = (int)((size_t)in.n_lc_vals / nv);
			if((size_t)in.n_lc_vals != nv * (size_t)fd)
				throw BackendError(E_SIZE, in.mask_vals ? "Wrong dimension for the user pointer array"
					: "Wrong dimension for the user pointer array (VectorField)");
			if(in.mask_vals && (size_t)in.n_mask_vals != nv)
				throw BackendError(E_SIZE, "Wrong dimension for the mask pointer array");
			if(fd != 3 && fd != 6)
				throw BackendError(E_SIZE, "Unexpected dimension for the LC orientational field, should be 3 or 6.");
			h->fd = fd;
			h->lc = in.lc_field_vals;
			h->G = (int)s.wavelengths.size();
			h->Nq = (int)s.q.size();
			h->spg = 2 * h->Nq;
			h->slots = h->G * h->spg;
			// ScreenOpticalFieldCollection (OpticalFieldCollection.cpp:37-39)
			long long need = (long long)h->slots * 2 * s.Nx * s.Ny;
			if((long long)in.n_E_vals != need)
				throw BackendError(E_SIZE, "Wrong dimension for the user pointer array (OpticalFieldCollection)");
			if(s.iso_thick.size() > 8) throw BackendError(E_SETTINGS, "At most 8 isotropic layers are supported");
			h->E = in.E_field_vals;
			if(in.mask_vals) {
				h->has_mask = true;
				mask_weights(s, in.mask_vals, in.mask_formula ? std::string(in.mask_formula) : std::string(),
					h->mask, h->wts);
				h->has_wts = false;
				for(double w : h->wts) if(w != 0.5) { h->has_wts = true; break; }
			}
			h->geom.Nx = s.Nx; h->geom.Ny = s.Ny; h->geom.N = s.Nx * s.Ny; h->geom.Nz = s.Nz;
			h->geom.spg = h->spg; h->geom.Nq = h->Nq;
			const double PI_REF = 3.1415926535897932;
			for(int g = 0; g < h->G; g++) {
				GroupParams gp;
				gp.wavelength = s.wavelengths[g];
				gp.k0 = 2 * PI_REF / gp.wavelength;
				gp.dX = gp.k0 * s.dx; gp.dY = gp.k0 * s.dy; gp.dZ = gp.k0 * s.dz;
				gp.no = s.no[g]; gp.ne = s.ne[g]; gp.ne_imag = s.ne_imag[g];
				gp.nhost = s.nhost[g]; gp.nin = s.nin[g];
				gp.nout_fresnel = s.iso_index.size() > 0 ? s.iso_index[0] : s.nout[g];
				gp.absorp_im = gp.ne_imag / (gp.ne - gp.no);
				gp.nref = 0;
				h->gps.push_back(gp);
			}
			for(auto& q : s.q) {
				if(!(q.first == 0 && q.second == 0)) h->any_shift = true;
				else h->any_zero_q = true;
			}
			ScreenParams& sp = h->sp;
			sp.Nx = s.Nx; sp.Ny = s.Ny; sp.Nq = h->Nq; sp.n_iso = (int)s.iso_thick.size();
			sp.dx = s.dx; sp.dy = s.dy; sp.NA = s.NA;
			// ScreenOutput ctor (ScreenOutput.cpp:32-38): z_foc -= t_p * nout(0.6) / n_p
			double zf = s.z_foc;
			for(size_t l = 0; l < s.iso_thick.size(); l++) zf -= s.iso_thick[l] * s.nout_06 / s.iso_index[l];
			sp.z_foc = zf;
			for(int l = 0; l < 8; l++) sp.thick[l] = l < sp.n_iso ? s.iso_thick[l] : 0;
			for(int l = 0; l < 9; l++) sp.index[l] = l < sp.n_iso ? s.iso_index[l] : 1;
			if(s.bulk_activate) {
				h->bulk = true;
				h->bulk_data.assign((size_t)h->slots * 2 * 3 * (size_t)s.Nx * s.Ny * s.Nz, 0.0);
			}
			h->index = (int)S.size();
			S.push_back(std::move(h));
		}
	}

	// Device memory the plan will hold, from the host-side settings alone.
	long long estimate_bytes() override {
		dry = true;
		allocate();
		dry = false;
		long long b = dev_bytes;
		dev_bytes = 0;
		scfg.clear();
		return b;
	}

	void setup(int ns, const nbpm_sample* samples) {
		setup_host(ns, samples);
		setup_device();
	}

	void setup_device() override {
		// Host-side validation is complete; only now touch the device.
		CK(cudaSetDevice(opt.device));
		CK(cudaStreamCreateWithFlags(&stream0, cudaStreamNonBlocking));
		CK(cudaStreamCreateWithFlags(&streamB0, cudaStreamNonBlocking));
		CK(cudaEventCreateWithFlags(&eBatch, cudaEventDisableTiming));
		for(auto& hp : S) {
			auto& L = hp->lane;
			if(hp->index == 0) { L.main = stream0; L.setup = streamB0; }
			else {
				L.owns_streams = true;
				CK(cudaStreamCreateWithFlags(&L.main, cudaStreamNonBlocking));
				CK(cudaStreamCreateWithFlags(&L.setup, cudaStreamNonBlocking));
			}
			for(cudaEvent_t* e : L.events()) CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
		}
		select(*S[0]);
		for(auto& e : ev) CK(cudaEventCreate(&e));
		int dev = opt.device;
		int optin = 0;
		CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
		smem_limit = (size_t)optin;
		CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
		CK(cudaFuncSetAttribute(k_fft_lines<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_limit));
		CK(cudaFuncSetAttribute(k_factor_chunked<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)((size_t)16 * 32 * 8 * sizeof(cx<R>) + 64 * sizeof(cx<R>))));
		CK(cudaFuncSetAttribute(k_shift_fused<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)((size_t)4 * (SHT + 6) * (SHT + 6) * sizeof(cx<R>))));
		if(sizeof(R) == sizeof(float)) {
			set_solve_smem_x_f32((int)smem_limit); set_solve_smem_y_f32((int)smem_limit); set_solve_smem_yt_f32((int)smem_limit);
			set_solve_smem_xs_f32((int)smem_limit); set_solve_smem_xw_f32((int)smem_limit);
		}
		else {
			set_solve_smem_x_f64((int)smem_limit); set_solve_smem_y_f64((int)smem_limit); set_solve_smem_yt_f64((int)smem_limit);
			set_solve_smem_xs_f64((int)smem_limit); set_solve_smem_xw_f64((int)smem_limit);
		}
		CK(cudaGetLastError());
		allocate();
		choose_configs();
	}

	int gpp(const SampleHost& h) const {
		int g = opt.groups_per_pass <= 0 ? h.G : std::min(opt.groups_per_pass, h.G);
		return std::max(1, g);
	}

	// Sizes every device buffer; with dry set, only adds up the bytes (admission estimates).
	bool dry = false;
	void dalloc(DevBuf& b, size_t bytes) {
		if(dry) b.bytes = bytes;
		else b.alloc(bytes);
	}

	// The frame in which the y-lines are x-lines (x' = y, y' = x).
	static Geom transposed(const Geom& G) {
		Geom t = G;
		t.Nx = G.Ny; t.Ny = G.Nx;
		return t;
	}

	SolveShape shape_of(const SampleHost& h) const {
		SolveShape sh;
		sh.Nx = h.s.Nx; sh.Ny = h.s.Ny; sh.spg = h.spg; sh.ng = gpp(h); sh.nw = h.s.n_woodbury;
		sh.fp32 = sizeof(R) == sizeof(float); sh.nsm = nsm;
		if(smem_limit) sh.smem = smem_limit;
		return sh;
	}

	void allocate() {
		scfg.clear();
		dev_bytes = 0;
		for(auto& hp : S) {
			SampleHost& h = *hp;
			size_t N = h.geom.N;
			int ng = gpp(h);
			const SolveShape sh = shape_of(h);
			SolveCfg sc = heuristic(sh);
			// buffers sized for every candidate the tuner may pick
			size_t px = sc.plane_x;
			for(auto& c : x_candidates(sh, true)) px = std::max(px, c.plane_x);
			sc.plane_x = px;
			bool need_t3 = sc.ys, need_t = sc.Mxt > 0;
			size_t py = sc.plane_y;
			for(auto& c : y_candidates(sh, true)) { need_t3 |= c.ys; need_t |= c.Mxt > 0; py = std::max(py, c.plane_y); }
			sc.plane_y = py;
			scfg.push_back(sc);
			// the sample's workspace (its lane)
			{
				auto& L = h.lane;
				const size_t nT = (size_t)ng * h.spg * 2 * N, nFx = (size_t)ng * 2 * NFAC * std::max(sc.plane_x, sc.plane_y);
				const size_t nL = (size_t)ng * 2 * std::max(h.s.Nx, h.s.Ny) * 2;
				dalloc(L.T, sizeof(cx<R>) * nT);
				dalloc(L.T2, sizeof(cx<R>) * nT);
				if(need_t3) dalloc(L.T3, sizeof(cx<R>) * nT);
				dalloc(L.Qring, sizeof(R) * (size_t)2 * ng * NQ * N);
				dalloc(L.coef, sizeof(cx<R>) * (size_t)2 * ng * coef_set_size((int)N));  // two slabs (transition kernels)
				dalloc(L.diag, sizeof(cx<R>) * (size_t)ng * NDIAG * N);
				if(need_t) {
					dalloc(L.coefT, sizeof(cx<R>) * (size_t)2 * ng * coef_set_size((int)N));
					dalloc(L.diagT, sizeof(cx<R>) * (size_t)ng * NDIAG * N);
				}
				L.facx_half = L.facy_half = nFx;
				L.lsc_half = nL;
				dalloc(L.facx, sizeof(cx<R>) * nFx * 2);
				dalloc(L.facy, sizeof(cx<R>) * nFx * 2);
				dalloc(L.lscx, sizeof(cx<double>) * nL * 2);
				dalloc(L.lscy, sizeof(cx<double>) * nL * 2);
				dalloc(L.scr, sizeof(cx<R>) * (size_t)2 * ng * 2 * 2 * N);  // x and y halves
				if(sizeof(R) != sizeof(double)) dalloc(L.stage, sizeof(cx<double>) * (size_t)h.slots * 2 * N);
				for(DevBuf* b : {&L.T, &L.T2, &L.T3, &L.Qring, &L.coef, &L.diag, &L.facx, &L.facy, &L.lscx, &L.lscy,
						&L.scr, &L.stage, &L.coefT, &L.diagT})
					dev_bytes += b->bytes;
			}
			// per-sample buffers
			dalloc(h.dir, sizeof(double) * h.nvox * h.fd);
			if(h.has_mask) dalloc(h.dmask, h.nvox);
			if(h.has_wts) dalloc(h.dwts, sizeof(double) * h.wts.size());
			dalloc(h.F, sizeof(cx<R>) * (size_t)h.slots * 2 * N);
			if(h.s.beam_type == 2) dalloc(h.E0, sizeof(cx<R>) * (size_t)h.slots * 2 * N);
			dalloc(h.gpsd, sizeof(GroupParams) * h.G);
			dalloc(h.shiftd, sizeof(ShiftParams) * h.G * h.Nq);
			dalloc(h.partial, sizeof(double) * h.G * 1024);
			dalloc(h.wl, sizeof(double) * h.G);
			dalloc(h.nout, sizeof(double) * h.G);
			dalloc(h.qv, sizeof(double) * 2 * h.Nq);
			if(h.bulk) {
				size_t nb = sizeof(cx<double>) * (size_t)ng * h.spg * 2 * N;
				dalloc(h.bstage, nb);
				dev_bytes += h.bstage.bytes;
				if(!dry && !h.hstage) CK(cudaMallocHost(reinterpret_cast<void**>(&h.hstage), nb));
			}
			dev_bytes += h.dir.bytes + h.dmask.bytes + h.dwts.bytes + h.F.bytes + h.E0.bytes;
			if(dry) dev_bytes += sizeof(cx<R>) * (size_t)(h.s.Nx + h.s.Ny);
			else { twiddles(h.s.Nx); twiddles(h.s.Ny); }
		}
	}

	// ---- line-solve configuration: forced, tuned or rule-based ----
	void choose_configs() {
		tune_notes.assign(S.size(), std::string());
		const std::string forced = opt.solve_config ? std::string(opt.solve_config) : std::string();
		bool zeroed = false;
		for(auto& hp : S) {
			SampleHost& h = *hp;
			const SolveShape sh = shape_of(h);
			SolveCfg& sc = scfg[h.index];
			const size_t pmax = sc.plane_x;
			const auto xc = x_candidates(sh), yc = y_candidates(sh);
			if(!forced.empty()) {
				const auto xr = x_candidates(sh, true), yr = y_candidates(sh, true);
				size_t k = forced.find(';');
				std::string fx = forced.substr(0, k), fy = k == std::string::npos ? "auto" : forced.substr(k + 1);
				auto pick = [&](const std::vector<SolveCfg>& cands, const std::string& want, bool x) {
					for(auto& c : cands) if((x ? c.xstr() : c.ystr()) == want) { if(x) sc.set_x(c); else sc.set_y(c); return; }
					std::string all;
					for(auto& c : cands) all += (all.empty() ? "" : ", ") + (x ? c.xstr() : c.ystr());
					throw BackendError(E_ARG, "solve configuration '" + want + "' is not a candidate for the " +
						std::to_string(h.s.Nx) + "x" + std::to_string(h.s.Ny) + " mesh with " + std::to_string(h.spg) +
						" slots per wavelength (candidates: " + all + ")");
				};
				if(fx != "auto") pick(xr, fx, true);
				if(fy != "auto") pick(yr, fy, false);
				if(sc.Mxt && !sc.x_hands_over())
					throw BackendError(E_ARG, "solve configuration '" + forced + "': the transposed-frame y solves (yx) need "
						"the x-lines on a kernel that hands the fields over (xc or xw)");
				tune_notes[h.index] = "forced";
				if(fx != "auto" && fy != "auto") { sc.plane_x = pmax; continue; }
			}
			if(opt.tune == 0 || (xc.size() <= 1 && yc.size() <= 1)) {
				if(tune_notes[h.index].empty()) tune_notes[h.index] = "rule-based";
				sc.plane_x = pmax;
				continue;
			}
			if(!zeroed) { zero_workspace(); zeroed = true; }
			const std::string key = tune_key(h);
			std::string note;
			for(int dirn = 0; dirn < 2; dirn++) {
				if(!forced.empty() && (dirn == 0 ? forced.substr(0, forced.find(';')) != "auto"
						: (forced.find(';') != std::string::npos && forced.substr(forced.find(';') + 1) != "auto")))
					continue;
				const auto& cands = dirn == 0 ? xc : yc;
				std::string hit;
				if(tune_cache_get((dirn == 0 ? "x|" : "y|") + key, hit)) {
					for(auto& c : cands)
						if((dirn == 0 ? c.xstr() : c.ystr()) == hit) { if(dirn == 0) sc.set_x(c); else sc.set_y(c); }
					note += std::string(dirn == 0 ? "x" : "y") + " cached " + hit + "; ";
					continue;
				}
				const SolveCfg keep = sc;
				double best = 1e300;
				SolveCfg win = sc;
				std::string times;
				for(auto& c : cands) {
					if(dirn == 1 && c.Mxt && !keep.x_hands_over()) continue;
					SolveCfg t = keep;
					if(dirn == 0) t.set_x(c); else t.set_y(c);
					t.plane_x = pmax;
					sc = t;
					double ms = time_direction(h, dirn);
					char b[96];
					std::snprintf(b, sizeof b, "%s %.3f ms", (dirn == 0 ? c.xstr() : c.ystr()).c_str(), ms);
					times += (times.empty() ? "" : ", ") + std::string(b);
					if(ms < best) { best = ms; win = t; }
				}
				sc = win;
				const std::string ws = dirn == 0 ? win.xstr() : win.ystr();
				tune_cache_put((dirn == 0 ? "x|" : "y|") + key, ws);
				note += std::string(dirn == 0 ? "x" : "y") + " tuned " + ws + " [" + times + "]; ";
			}
			sc.plane_x = pmax;
			tune_notes[h.index] = (tune_notes[h.index].empty() ? "" : tune_notes[h.index] + ", ") + note;
			if(opt.verbose) std::printf("line solves %s: %s\n", sc.str().c_str(), note.c_str());
		}
		launches = 0;
		// the scratch field of the scratch-chunk y solve is kept only where that solve was chosen
		for(auto& hp : S) {
			auto& L = hp->lane;
			auto drop = [&](DevBuf& b) { dev_bytes -= (long long)b.bytes; b.alloc(0); };
			if(!scfg[hp->index].ys && L.T3.p) drop(L.T3);
			if(!scfg[hp->index].Mxt && L.coefT.p) { drop(L.coefT); drop(L.diagT); }
		}
		select(*S[0]);
	}

	// Wavelengths per pass the tuner times with (and keys on): at most four. Beyond that every
	// candidate's grid already fills the device many times over, the ranking does not change, and
	// timing fewer wavelengths keeps the tuning of large plans (serving: many shapes) short.
	int tune_groups(const SampleHost& h) const { return std::min(gpp(h), 4); }

	std::string tune_key(const SampleHost& h) const {
		char b[160];
		std::snprintf(b, sizeof b, "%s|%dx%d|spg%d|ng%d|nw%d|sm%d", sizeof(R) == sizeof(float) ? "fp32" : "fp64", h.s.Nx,
			h.s.Ny, h.spg, tune_groups(h), h.s.n_woodbury, nsm);
		return b;
	}

	// Zeroes the workspace the timing runs read (their values do not change the kernels' speed,
	// but uninitialised memory could hold NaN or denormal patterns).
	void zero_workspace() {
		for(auto& hp : S) {
			auto& L = hp->lane;
			for(DevBuf* b : {&L.T, &L.T2, &L.T3, &L.coef, &L.facx, &L.facy, &L.lscx, &L.lscy, &L.coefT, &L.diagT, &hp->F})
				if(b->p) CK(cudaMemsetAsync(b->p, 0, b->bytes, stream0));
		}
		CK(cudaStreamSynchronize(stream0));
	}

	// Device time of one slab's solves of one direction with the current configuration of
	// sample h (explicit step + Woodbury iterates, eager launches on the main stream): the best of
	// three runs after one warm-up.
	double time_direction(SampleHost& h, int dirn) {
		const Geom Gm = h.geom;
		const int ng = tune_groups(h), nsl = ng * h.spg;
		cx<R>* Fp = h.F.as<cx<R>>();
		select(h);
		fx_cur = W->facx.as<cx<R>>(); fy_cur = W->facy.as<cx<R>>();
		lx_cur = W->lscx.as<cx<double>>(); ly_cur = W->lscy.as<cx<double>>();
		ct_cur = W->coefT.as<cx<R>>();
		float best = 1e30f;
		for(int r = 0; r < 4; r++) {
			CK(cudaEventRecord(ev[2], stream));
			rec_adi(h, Gm, 0, nsl, ng, h.s.n_woodbury, W->coef.as<cx<R>>(), Fp, W->T.as<cx<R>>(), W->T2.as<cx<R>>(), Fp, dirn);
			CK(cudaEventRecord(ev[3], stream));
			CK(cudaEventSynchronize(ev[3]));
			float ms = 0;
			CK(cudaEventElapsedTime(&ms, ev[2], ev[3]));
			if(r > 0) best = std::min(best, ms);
		}
		return best;
	}

	void upload() override {
		for(auto& hp : S) {
			SampleHost& h = *hp;
			select(h);
			CK(cudaMemcpyAsync(h.dir.p, h.lc, h.dir.bytes, cudaMemcpyHostToDevice, stream));
			if(h.has_mask) CK(cudaMemcpyAsync(h.dmask.p, h.mask.data(), h.nvox, cudaMemcpyHostToDevice, stream));
			if(h.has_wts) CK(cudaMemcpyAsync(h.dwts.p, h.wts.data(), h.dwts.bytes, cudaMemcpyHostToDevice, stream));
			CK(cudaMemcpyAsync(h.gpsd.p, h.gps.data(), h.gpsd.bytes, cudaMemcpyHostToDevice, stream));
			CK(cudaMemcpyAsync(h.wl.p, h.s.wavelengths.data(), h.wl.bytes, cudaMemcpyHostToDevice, stream));
			CK(cudaMemcpyAsync(h.nout.p, h.s.nout.data(), h.nout.bytes, cudaMemcpyHostToDevice, stream));
			std::vector<double> qflat;
			for(auto& q : h.s.q) { qflat.push_back(q.first); qflat.push_back(q.second); }
			CK(cudaMemcpyAsync(h.qv.p, qflat.data(), h.qv.bytes, cudaMemcpyHostToDevice, stream));
			CK(cudaStreamSynchronize(stream));  // qflat lifetime
			if(h.s.beam_type == 2) {
				size_t n = (size_t)h.slots * 2 * h.geom.N;
				if(sizeof(R) == sizeof(double)) {
					CK(cudaMemcpyAsync(h.E0.p, h.E, n * sizeof(cx<double>), cudaMemcpyHostToDevice, stream));
				}
				else {
					CK(cudaMemcpyAsync(W->stage.p, h.E, n * sizeof(cx<double>), cudaMemcpyHostToDevice, stream));
					k_narrow<R><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, W->stage.as<cx<double>>(), h.E0.as<cx<R>>());
					CK(cudaGetLastError());
				}
			}
			CK(cudaStreamSynchronize(stream));
		}
		select(*S[0]);
	}

	// Device address of a page-locked, mapped host buffer of the given size (the caller's result
	// array), or null. Both ends of the range must be mapped with one contiguous device mapping,
	// so that a kernel writing the whole array through it stays inside the mapped range.
	static void* mapped_host(void* p, size_t bytes) {
		if(!bytes) return nullptr;
		cudaPointerAttributes a, b;
		if(cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return nullptr; }
		if(a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
		char* last = static_cast<char*>(p) + bytes - 1;
		if(cudaPointerGetAttributes(&b, last) != cudaSuccess) { cudaGetLastError(); return nullptr; }
		if(b.type != cudaMemoryTypeHost || !b.devicePointer) return nullptr;
		if(static_cast<char*>(b.devicePointer) - static_cast<char*>(a.devicePointer) != (ptrdiff_t)(bytes - 1)) return nullptr;
		return a.devicePointer;
	}

	void download() override {
		for(auto& hp : S) {
			SampleHost& h = *hp;
			select(h);
			size_t n = (size_t)h.slots * 2 * h.geom.N;
			void* dE = mapped_host(h.E, n * sizeof(cx<double>));
			if(sizeof(R) == sizeof(double) && dE) {
				// page-locked result array: copied by a kernel through the mapping
				k_copy<R><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, h.F.as<cx<R>>(), static_cast<cx<R>*>(dE));
				CK(cudaGetLastError());
			}
			else if(sizeof(R) == sizeof(double)) {
				CK(cudaMemcpyAsync(h.E, h.F.p, n * sizeof(cx<double>), cudaMemcpyDeviceToHost, stream));
			}
			else if(dE) {
				// page-locked result array: the widening kernel writes it directly
				k_widen<R><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, h.F.as<cx<R>>(), static_cast<cx<double>*>(dE));
				CK(cudaGetLastError());
			}
			else {
				k_widen<R><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, h.F.as<cx<R>>(), W->stage.as<cx<double>>());
				CK(cudaGetLastError());
				CK(cudaMemcpyAsync(h.E, W->stage.p, n * sizeof(cx<double>), cudaMemcpyDeviceToHost, stream));
			}
		}
		for(auto& hp : S) CK(cudaStreamSynchronize(hp->lane.main));
		select(*S[0]);
		host_finish();
	}

	bool reusable() const override {
		for(auto& hp : S)
			if(hp->bulk) return false;
		return true;
	}
	// Returns false (nothing changed) when the call needs another recording: other sizes, or
	// mask weights that switch between uniform and formula-derived.
	bool rebind(int ns, const nbpm_sample* samples) override {
		if(ns != (int)S.size()) return false;
		// a device reset since the plan was made leaves its buffers unknown to the runtime
		{
			cudaPointerAttributes a;
			if(cudaPointerGetAttributes(&a, S[0]->F.p) != cudaSuccess || a.type != cudaMemoryTypeDevice) {
				cudaGetLastError();
				return false;
			}
		}
		std::vector<std::vector<unsigned char>> masks(ns);
		std::vector<std::vector<double>> wts(ns);
		for(int i = 0; i < ns; i++) {
			SampleHost& h = *S[i];
			const nbpm_sample& in = samples[i];
			if(!in.lc_field_vals || !in.E_field_vals) throw BackendError(E_ARG, "null pointer argument");
			if((size_t)in.n_lc_vals != h.nvox * (size_t)h.fd || (long long)in.n_E_vals != (long long)h.slots * 2 * h.geom.N ||
					(in.mask_vals != nullptr) != h.has_mask)
				return false;
			if(in.mask_vals) {
				if((size_t)in.n_mask_vals != h.nvox) return false;
				mask_weights(h.s, in.mask_vals, in.mask_formula ? std::string(in.mask_formula) : std::string(), masks[i], wts[i]);
				bool nonuniform = false;
				for(double w : wts[i]) if(w != 0.5) { nonuniform = true; break; }
				if(nonuniform != h.has_wts) return false;
			}
		}
		for(int i = 0; i < ns; i++) {
			SampleHost& h = *S[i];
			h.lc = samples[i].lc_field_vals;
			h.E = samples[i].E_field_vals;
			if(h.has_mask) { h.mask.swap(masks[i]); h.wts.swap(wts[i]); }
		}
		return true;
	}

	// Host-side outputs of a finished run: the bulk-output files.
	void host_finish() override {
		for(auto& hp : S)
			if(hp->bulk) write_bulk(*hp);
	}

	// ---- launch helpers (count launches while recording) ----
	dim3 pgrid(int N, int ny, int threads = 256) { return dim3((unsigned)((N + threads - 1) / threads), (unsigned)ny); }

	void fft2(SampleHost& h, cx<R>* F, int nplanes, int sign) {
		int Nx = h.s.Nx, Ny = h.s.Ny;
		for(int pass = 0; pass < 2; pass++) {
			int n = pass == 0 ? Nx : Ny;
			if(n == 1) continue;
			FftPlan1D P;
			if(!fft_plan_1d(n, P)) throw BackendError(E_INTERNAL, "FFT plan too deep");
			size_t per_line = 2 * (size_t)(n + 1) * sizeof(cx<R>);
			if(per_line > smem_limit)
				throw BackendError(E_SETTINGS, "FFT line length " + std::to_string(n) + " exceeds shared memory");
			int lpb = (int)std::max<size_t>(1, std::min<size_t>(64, (size_t)(48 * 1024) / per_line));
			if(pass == 1) lpb = std::max(lpb, std::min(16, (int)(smem_limit / per_line)));
			lpb = std::max(1, std::min(lpb, (int)(smem_limit / per_line)));
			size_t smem = per_line * lpb;
			int nlines, lpp;
			long long ps = (long long)Nx * Ny, ls, es;
			if(pass == 0) { nlines = nplanes * Ny; lpp = Ny; ls = Nx; es = 1; }
			else { nlines = nplanes * Nx; lpp = Nx; ls = 1; es = Nx; }
			int blocks = (nlines + lpb - 1) / lpb;
			int threads = std::min(256, std::max(32, ((lpb * n / 2) + 31) / 32 * 32));
			cx<R>* tw = twiddles(n);
			double bytes = 2.0 * sizeof(cx<R>) * (double)nplanes * Nx * Ny;
			launch(pass == 0 ? "fft_rows" : "fft_cols", bytes, [&] {
				k_fft_lines<R><<<blocks, threads, smem, cs>>>(F, nullptr, P, nlines, lpp, ps, ls, es, lpb, tw, sign);
			});
		}
	}

	// Every sample on its own lane: the lanes of samples 1.. fork from the plan's stream and join
	// it again at the end, so that in the captured graph the samples are parallel branches.
	void record() {
		launches = 0;
		select(*S[0]);
		if(S.size() > 1) CK(cudaEventRecord(eBatch, stream0));
		for(auto& hp : S) {
			select(*hp);
			if(hp->index > 0) CK(cudaStreamWaitEvent(stream, eBatch, 0));
			record_sample(*hp);
			if(hp->index > 0) CK(cudaEventRecord(hp->lane.eEnd, stream));
		}
		select(*S[0]);
		for(auto& hp : S)
			if(hp->index > 0) CK(cudaStreamWaitEvent(stream0, hp->lane.eEnd, 0));
	}

	// State of one pass of wavelength groups through the slab loop. Kept between calls when a
	// sample is advanced a few slabs at a time (serving), so that the launch sequence is the
	// same as in one uninterrupted recording.
	struct PassState {
		int ga = 0, ng = 0, slot0 = 0, nsl = 0;
		int iz = 0;  // next slab
		const GroupParams* gps = nullptr;
		cx<R>* Fp = nullptr;
		cx<R>* Tb = nullptr;
		cx<R>* T2b = nullptr;
		R* Qr[2] = {nullptr, nullptr};
		cx<R>* Cring[2] = {nullptr, nullptr};
		cx<R>* Dg = nullptr;
		const cx<R>* Cprev = nullptr;
		double eps_bytes = 0, field_pts = 0;
	};

	// nref of every group, then the shift parameters (device side). Runs on the setup stream,
	// overlapping the entrance of the first pass on the main stream; the first transition
	// waits for it (eNref).
	void rec_prologue(SampleHost& h) {
		const uint8_t* mk_ = h.has_mask ? h.dmask.as<uint8_t>() : nullptr;
		CK(cudaEventRecord(eNrefFork, stream));
		CK(cudaStreamWaitEvent(streamB, eNrefFork, 0));
		cs = streamB;
		int nb = (int)std::min<size_t>(1024, (h.nvox + 255) / 256);
		launch("neff_partial", (double)h.nvox * h.fd * 8 * h.G, [&] {
			k_neff_partial<sizeof(R) == sizeof(float)><<<dim3(nb, h.G), 256, 0, cs>>>(h.dir.as<double>(), h.fd, mk_, h.nvox,
				h.gpsd.as<GroupParams>(), h.partial.as<double>());
		});
		launch("nref_final", 8.0 * nb * h.G, [&] {
			k_nref_final<<<(h.G + 63) / 64, 64, 0, cs>>>(h.G, nb, h.nvox, h.partial.as<double>(),
				h.gpsd.as<GroupParams>());
		});
		launch("shift_params", sizeof(ShiftParams) * h.G * h.Nq, [&] {
			k_shift_params<<<(h.G * h.Nq + 63) / 64, 64, 0, cs>>>(h.G, h.Nq, h.geom.Nx, h.geom.Ny,
				h.gpsd.as<GroupParams>(), h.qv.as<double>(), h.shiftd.as<ShiftParams>());
		});
		CK(cudaEventRecord(eNref, streamB));
		cs = stream;
	}

	// Entrance of a pass: eps plane 0 and the initial fields.
	PassState rec_pass_begin(SampleHost& h, int ga) {
		const Geom Gm = h.geom;
		const int N = Gm.N;
		const double sc = sizeof(cx<R>);
		const uint8_t* mk_ = h.has_mask ? h.dmask.as<uint8_t>() : nullptr;
		PassState ps;
		ps.ga = ga;
		ps.ng = std::min(gpp(h), h.G - ga);
		ps.slot0 = ga * h.spg;
		ps.nsl = ps.ng * h.spg;
		ps.gps = h.gpsd.as<GroupParams>() + ga;
		ps.Fp = h.F.as<cx<R>>() + (size_t)ps.slot0 * 2 * N;
		ps.Tb = W->T.as<cx<R>>();
		ps.T2b = W->T2.as<cx<R>>();
		ps.Qr[0] = W->Qring.as<R>();
		ps.Qr[1] = ps.Qr[0] + (size_t)ps.ng * NQ * N;
		ps.Cring[0] = W->coef.as<cx<R>>();
		ps.Cring[1] = W->coef.as<cx<R>>() + (size_t)ps.ng * coef_set_size(N);
		ps.Dg = W->diag.as<cx<R>>();
		ps.eps_bytes = (double)N * ps.ng * (h.fd * 8 + (mk_ ? 1 : 0) + NQ * sizeof(R));
		ps.field_pts = (double)N * ps.nsl;
		const int ng = ps.ng, nsl = ps.nsl, slot0 = ps.slot0;
		const GroupParams* gps = ps.gps;
		launch("eps_plane", ps.eps_bytes, [&] {
			k_eps_plane<R><<<pgrid(N, ng), 256, 0, cs>>>(h.dir.as<double>(), h.fd, mk_, N, 0, gps, ps.Qr[0]);
		});
		if(h.s.beam_type != 2) {
			launch("init_fields", ps.field_pts * 2 * sc + (double)N * ng * 3 * 8, [&] {
				const double th1 = 0.5 * 3.1415926535897932;  // polarisation angle of pol = 1 (BPMIteration.cpp:87-109)
				k_init_fields<R><<<pgrid(N, nsl), 256, 0, cs>>>(Gm, slot0, gps, ps.Qr[0], h.s.beam_type,
					h.s.waist, h.s.dx, h.s.dy, std::cos(th1), std::sin(th1), ps.Fp);
			});
		}
		else {
			size_t n = (size_t)nsl * 2 * N;
			launch("copy_fields", 2.0 * n * sc, [&] {
				k_copy<R><<<(unsigned)((n + 255) / 256), 256, 0, cs>>>(n, h.E0.as<cx<R>>() + (size_t)slot0 * 2 * N, ps.Fp);
			});
		}
		return ps;
	}

	// Slabs [ps.iz, iz_end) of a pass. Setup of slab iz (eps plane iz+1, coefficients,
	// factorisations) runs on streamB and overlaps the right-hand-side work of slab iz-1 on
	// the main stream; both streams are joined again before returning.
	void rec_pass_slabs(SampleHost& h, PassState& ps, int iz_end) {
		const Geom Gm = h.geom;
		const int N = Gm.N, Nx = Gm.Nx, Ny = Gm.Ny;
		const int Nw = h.s.n_woodbury;
		const double sc = sizeof(cx<R>);
		const uint8_t* mk_ = h.has_mask ? h.dmask.as<uint8_t>() : nullptr;
		const double* wts = h.has_wts ? h.dwts.as<double>() : nullptr;
		const int ng = ps.ng, nsl = ps.nsl, slot0 = ps.slot0;
		const GroupParams* gps = ps.gps;
		if(ps.iz >= iz_end) return;
		CK(cudaStreamWaitEvent(stream, eNref, 0));  // shift parameters
		CK(cudaEventRecord(eFork, stream));
		CK(cudaStreamWaitEvent(streamB, eFork, 0));
		for(int iz = ps.iz; iz < iz_end; iz++) {
			R* QA = ps.Qr[iz & 1];
			R* QB = ps.Qr[(iz + 1) & 1];
			cx<R>* C = ps.Cring[iz & 1];
			const SolveCfg& scf = scfg[h.index];
			cx<R>* fx = W->facx.as<cx<R>>() + (size_t)(iz & 1) * W->facx_half;
			cx<R>* fy = W->facy.as<cx<R>>() + (size_t)(iz & 1) * W->facy_half;
			cx<double>* lx = W->lscx.as<cx<double>>() + (size_t)(iz & 1) * W->lsc_half;
			cx<double>* ly = W->lscy.as<cx<double>>() + (size_t)(iz & 1) * W->lsc_half;
			// ---- setup stream ----
			cs = streamB;
			launch("eps_plane", ps.eps_bytes, [&] {
				k_eps_plane<R><<<pgrid(N, ng), 256, 0, cs>>>(h.dir.as<double>(), h.fd, mk_, N, iz + 1, gps, QB);
			});
			// coef(iz) overwrites the set the transition of slab iz-1 read (slab iz-2)
			if(iz >= 1) CK(cudaStreamWaitEvent(streamB, eTrans, 0));
			launch("coef", (double)N * ng * (2 * NQ * sizeof(R) + NCOEF * sc + NDIAG * sc + (wts ? 16 : 0)), [&] {
				k_coef<R><<<pgrid(N, ng, 128), 128, 0, cs>>>(QA, QB, wts, iz, Gm, gps, C, ps.Dg);
			});
			CK(cudaEventRecord(eCoef, streamB));
			// factor(iz) overwrites the half the line solves of slab iz-2 used
			if(iz >= 2) CK(cudaStreamWaitEvent(streamB, eAdi[iz & 1], 0));
			const double fb = (double)N * ng * 2 * (3 * sc + NFAC * sc + 4 * sc);
			// y factorisation: 8 chunk warps per 32 columns, 16 when the grid leaves SMs idle
			const int LT = 4, WF = ((Nx + 31) / 32) * 2 * ng < nsm && Ny - 1 >= 256 ? 16 : 8;
			launch("factor_x", fb, [&] {
				k_factor_chunked<R, 0><<<dim3((unsigned)((Ny + LT - 1) / LT), (unsigned)(ng * 2)), dim3(32, LT), 0, cs>>>(
					Gm, ng, scf.Mx, 32 * scf.WPLx, 1, ps.Dg, fx, scf.plane_x, lx);
			});
			cx<R>* CT = scf.Mxt ? W->coefT.as<cx<R>>() + (size_t)(iz & 1) * ng * coef_set_size(N) : nullptr;
			if(scf.Mxt) {
				// y-lines as x-lines of the transposed frame: transposed coefficients and diagonals,
				// then the x-line factorisation of that frame
				const Geom Gt = transposed(Gm);
				launch("coef_t", 2.0 * N * ng * NCT * sc, [&] {
					k_coef_t<R><<<dim3((unsigned)((Nx + 31) / 32), (unsigned)((Ny + 31) / 32), (unsigned)(ng * NCT)), dim3(32, 8), 0,
						cs>>>(Gm, C, ps.Dg, CT, W->diagT.as<cx<R>>());
				});
				launch("factor_y", fb, [&] {
					k_factor_chunked<R, 0><<<dim3((unsigned)((Nx + LT - 1) / LT), (unsigned)(ng * 2)), dim3(32, LT), 0, cs>>>(
						Gt, ng, scf.Mxt, 32 * scf.WPLt, 1, W->diagT.as<cx<R>>(), fy, scf.plane_y, ly);
				});
			}
			else {
				size_t smem = (size_t)WF * 32 * 8 * sizeof(cx<R>) + 64 * sizeof(cx<R>);
				launch("factor_y", fb, [&] {
					k_factor_chunked<R, 1><<<dim3((unsigned)((Nx + 31) / 32), (unsigned)(ng * 2)), dim3(32, WF), smem, cs>>>(
						Gm, ng, 0, 32, WF, ps.Dg, fy, scf.plane_y, ly);
				});
			}
			CK(cudaEventRecord(eFac, streamB));
			// ---- main stream ----
			cs = stream;
			CK(cudaStreamWaitEvent(stream, eCoef, 0));
			// [phase(iz-1)] shift(iz-1) | shift(iz) phase(iz)   (BPMIteration.cpp:133-146)
			const cx<R>* xsrc = rec_transition(h, slot0, nsl, ps.Cprev, C, ps.Fp, ps.Tb, ps.T2b, iz > 0);
			CK(cudaEventRecord(eTrans, stream));
			CK(cudaStreamWaitEvent(stream, eFac, 0));
			fx_cur = fx; fy_cur = fy; lx_cur = lx; ly_cur = ly; ct_cur = CT;
			rec_adi(h, Gm, slot0, nsl, ng, Nw, C, ps.Fp, ps.Tb, ps.T2b, xsrc);
			rec_bulk(h, ps, iz + 1, C);
			CK(cudaEventRecord(eAdi[iz & 1], stream));
			ps.Cprev = C;
		}
		ps.iz = iz_end;
		CK(cudaEventRecord(eJoin, streamB));
		CK(cudaStreamWaitEvent(stream, eJoin, 0));
		cs = stream;
	}

	// Exit of a pass: the last slab's trailing phase and shift, then the Fresnel exit operator.
	void rec_pass_end(SampleHost& h, PassState& ps) {
		const Geom Gm = h.geom;
		const int N = Gm.N, Nz = Gm.Nz;
		const double sc = sizeof(cx<R>);
		cs = stream;
		CK(cudaStreamWaitEvent(stream, eNref, 0));
		if(Nz > 1) rec_transition(h, ps.slot0, ps.nsl, ps.Cprev, nullptr, ps.Fp, ps.Tb, ps.T2b, false);
		const GroupParams* gps = ps.gps;
		R* Qlast = ps.Qr[(Nz - 1) & 1];
		const int nsl = ps.nsl, slot0 = ps.slot0;
		launch("fresnel_out", ps.field_pts * 4 * sc + (double)N * ps.ng * 3 * 8, [&] {
			k_fresnel_out<R><<<pgrid(N, nsl), 256, 0, cs>>>(Gm, slot0, gps, Qlast, ps.Fp);
		});
	}

	// Screen filter over every plane of the sample (ScreenOutput.cpp:184-224).
	void rec_screen(SampleHost& h) {
		const int N = h.geom.N;
		const double sc = sizeof(cx<R>);
		cx<R>* F = h.F.as<cx<R>>();
		int nplanes = h.slots * 2;
		fft2(h, F, nplanes, -1);
		launch("screen_filter", (double)N * h.slots * 4 * sc, [&] {
			k_screen_filter<R><<<pgrid(N, h.G * h.Nq, 128), 128, 0, cs>>>(F, h.sp, 0, h.wl.as<double>(),
				h.nout.as<double>(), h.qv.as<double>());
		});
		fft2(h, F, nplanes, +1);
	}

	// Bulk output of plane iz of a pass (BPMIteration.cpp:111-121, 153-168). The entrance
	// plane (C null) is the current field; plane iz >= 1 is the field after the slab's
	// trailing phase and shift, which the slab loop defers to the next transition, so it is
	// formed out of place here.
	std::deque<BulkRec> bulk_recs;
	void rec_bulk(SampleHost& h, PassState& ps, int iz, const cx<R>* C) {
		if(!h.bulk) return;
		const Geom Gm = h.geom;
		const int N = Gm.N;
		const size_t n = (size_t)ps.nsl * 2 * N;
		const double sc = sizeof(cx<R>);
		cx<double>* st = h.bstage.as<cx<double>>();
		const cx<R>* src = ps.Fp;
		cs = stream;
		if(C) {
			cx<R>* o = sizeof(R) == sizeof(double) ? reinterpret_cast<cx<R>*>(st) : ps.T2b;
			dim3 grid((unsigned)((Gm.Nx + SHT - 1) / SHT), (unsigned)((Gm.Ny + SHT - 1) / SHT), (unsigned)ps.nsl);
			size_t smem = (size_t)4 * (SHT + 6) * (SHT + 6) * sizeof(cx<R>);
			launch("bulk_plane", (double)n * 2 * sc, [&] {
				k_shift_fused<R><<<grid, 256, smem, cs>>>(Gm, ps.slot0, h.shiftd.as<ShiftParams>(), C, nullptr, 1, ps.Fp, o);
			});
			src = o;
		}
		if(reinterpret_cast<const void*>(src) != reinterpret_cast<const void*>(st)) {
			launch("bulk_widen", (double)n * (sc + 16), [&] {
				k_widen<R><<<(unsigned)((n + 255) / 256), 256, 0, cs>>>(n, src, st);
			});
		}
		CK(cudaMemcpyAsync(h.hstage, st, n * sizeof(cx<double>), cudaMemcpyDeviceToHost, cs));
		bulk_recs.push_back(BulkRec{&h, ps.slot0, ps.nsl, iz});
		CK(cudaLaunchHostFunc(cs, bulk_host_fn, &bulk_recs.back()));
	}

	void write_bulk(SampleHost& h) {
		const auto& s = h.s;
		const size_t NV = (size_t)s.Nx * s.Ny * s.Nz;
		std::vector<VtiArray> fd, pd;
		std::vector<double> qx, qy;
		for(auto& q : s.q) { qx.push_back(q.first); qy.push_back(q.second); }
		fd.push_back({"lambda", 1, s.wavelengths.data(), s.wavelengths.size()});
		fd.push_back({"qx", 1, qx.data(), qx.size()});
		fd.push_back({"qy", 1, qy.data(), qy.size()});
		const char* pols[2] = {"inputX_", "inputY_"};
		for(int w = 0; w < h.G; w++)
			for(int q = 0; q < h.Nq; q++)
				for(int pol = 0; pol < 2; pol++) {
					size_t slot = (size_t)pol + 2 * ((size_t)q + (size_t)h.Nq * w);
					const double* re = h.bulk_data.data() + slot * 2 * 3 * NV;
					std::string tag = std::string(pols[pol]) + std::to_string(q) + "_" + std::to_string(w);
					pd.push_back({"E_real_" + tag, 3, re, NV});
					pd.push_back({"E_imag_" + tag, 3, re + 3 * NV, NV});
				}
		std::string path = bulk_output_path(s.results_folder, s.bulk_base_name);
		if(opt.verbose) std::printf("Exporting bulk optical field to %s\n", path.c_str());
		std::string err = write_vti(path, s.Nx, s.Ny, s.Nz, s.dx, s.dy, s.dz, fd, pd);
		if(!err.empty()) throw BackendError(E_INTERNAL, "bulk output: " + err);
	}

	void record_sample(SampleHost& h) {
		rec_prologue(h);
		for(int ga = 0; ga < h.G; ga += gpp(h)) {
			PassState ps = rec_pass_begin(h, ga);
			rec_bulk(h, ps, 0, nullptr);
			rec_pass_slabs(h, ps, h.geom.Nz - 1);
			rec_pass_end(h, ps);
		}
		rec_screen(h);
	}

	// Between the Strang half-steps of consecutive slabs: phase(CA) -> shift -> [shift] ->
	// phase(CB), with CA / CB the coefficient sets of the previous / current slab (null: no
	// phase) and two_shifts selecting shift(iz-1) followed by shift(iz). If every slot is at
	// q = 0 the shifts reduce to the duplicate-border copy and the whole transition is one pass.
	// Returns where the transitioned field is: Fp, or T2b when the one-pass kernel ran (only
	// before a fused x-solve, which then reads it from there).
	const cx<R>* rec_transition(SampleHost& h, int slot0, int nsl, const cx<R>* CA, const cx<R>* CB, cx<R>* Fp,
			cx<R>* Tb, cx<R>* T2b, bool two_shifts) {
		const Geom Gm = h.geom;
		const double sc = sizeof(cx<R>);
		const double fpb = (double)Gm.N * nsl * 4 * sc;
		const ShiftParams* sp = h.shiftd.as<ShiftParams>();
		if(!h.any_shift) {
			launch("phase_sync", fpb, [&] {
				k_phase_sync<R><<<pgrid(Gm.N, nsl), 256, 0, cs>>>(Gm, slot0, CA, CB, Fp);
			});
			return Fp;
		}
		if(CB && scfg[h.index].Mx > 0) {
			const int nsh = two_shifts ? 2 : 1;
			dim3 grid((unsigned)((Gm.Nx + SHT - 1) / SHT), (unsigned)((Gm.Ny + SHT - 1) / SHT), (unsigned)nsl);
			size_t smem = (size_t)4 * (SHT + 6) * (SHT + 6) * sizeof(cx<R>);
			launch("shift_fused", fpb + (double)Gm.N * (nsl / Gm.spg) * 6 * sc, [&] {
				k_shift_fused<R><<<grid, 256, smem, cs>>>(Gm, slot0, sp, CA, CB, nsh, Fp, T2b);
			});
			return T2b;
		}
		launch("shift_x", fpb, [&] {
			k_shift_x<R><<<pgrid(Gm.N, nsl), 256, 0, cs>>>(Gm, slot0, sp, CA, Fp, T2b);
		});
		if(two_shifts) {
			launch("shift_y", fpb, [&] {
				k_shift_y<R><<<pgrid(Gm.N, nsl), 256, 0, cs>>>(Gm, slot0, sp, nullptr, T2b, Tb);
			});
			launch("shift_x", fpb, [&] {
				k_shift_x<R><<<pgrid(Gm.N, nsl), 256, 0, cs>>>(Gm, slot0, sp, nullptr, Tb, T2b);
			});
		}
		launch("shift_y", fpb, [&] {
			k_shift_y<R><<<pgrid(Gm.N, nsl), 256, 0, cs>>>(Gm, slot0, sp, CB, T2b, Fp);
		});
		return Fp;
	}

	// Sequential line solve (lines too long for the chunked kernels).
	void rec_solve_seq(int dirn, SampleHost& h, const Geom& Gm, int slot0, int nsl, int ng, const cx<R>* src,
			cx<R>* dst, const cx<R>* acc_in, cx<R>* acc_out) {
		const SolveCfg& sc = scfg[h.index];
		int nlines = dirn == 0 ? Gm.Ny : Gm.Nx;
		int nt = nsl * 2 * nlines;
		const double sz = sizeof(cx<R>);
		double bytes = (double)Gm.N * nsl * 2 * sz * (acc_out ? 4 : 2) + (double)Gm.N * ng * 2 * NFAC * sz;
		if(dirn == 0)
			launch("solve_x", bytes, [&] {
				k_solve<R, 0><<<(nt + 127) / 128, 128, 0, cs>>>(Gm, slot0, nsl, fx_cur, sc.plane_x, lx_cur, src, dst,
					acc_in, acc_out);
			});
		else
			launch("solve_y", bytes, [&] {
				k_solve<R, 1><<<(nt + 127) / 128, 128, 0, cs>>>(Gm, slot0, nsl, fy_cur, sc.plane_y, ly_cur, src, dst,
					acc_in, acc_out);
			});
	}

	// Fused right-hand side + chunked line solve. wood = false: explicit half-step of the other
	// direction; wood = true: Woodbury term. dst may be null (t not needed afterwards).
	// Whether the fused solve of direction dirn runs k_solve_xc / k_solve_yc, the kernels that take
	// a second accumulator input.
	bool solve_takes_acc2(const SolveCfg& sc, int dirn) const {
		return dirn == 0 ? (sc.Mx > 0 && !sc.xs) : (sc.yq > 0 || sc.Mt > 0 || sc.Mxt > 0 || (sc.My > 0 && !sc.ys));
	}

	// scr: a field-sized buffer the solve may overwrite (none of src, acc_in, acc_in2), used by the
	// sequential y solve for its forward values.
	// tout: k_solve_xc writes its results transposed with the components exchanged (the hand-over
	// between the x frame and the transposed frame of the y solves).
	void rec_solve_fused(int dirn, bool wood, SampleHost& h, const Geom& Gm, int slot0, int nsl, int ng,
			const cx<R>* C, const cx<R>* src, cx<R>* dst, const cx<R>* acc_in, cx<R>* acc_out,
			const cx<R>* acc_in2, cx<R>* scr, bool tout = false) {
		const SolveCfg& sc = scfg[h.index];
		const double sz = sizeof(cx<R>);
		double fp = (double)Gm.N * nsl * 2 * sz;
		// algorithmic bytes: every distinct field read once (an accumulator input that is the
		// source itself is not read twice), every field written once, coefficients and factors
		// once per wavelength
		const int reads = 1 + (acc_in && acc_in != src ? 1 : 0) + (acc_in2 && acc_in2 != src && acc_in2 != acc_in ? 1 : 0);
		const int writes = (dst ? 1 : 0) + (acc_out ? 1 : 0);
		double bytes = fp * (reads + writes) + (double)Gm.N * ng * (2 * NFAC + (wood ? 14 : 20)) * sz;
		SolveLaunch L;
		L.stream = cs;
		if(dirn == 0) {
			L.M = sc.Mx; L.kind = wood ? ST_WOOD_X : ST_EXPL_Y;
			const int LT = 4;
			L.KS = sc.KSx;
			int nch = h.spg / L.KS;
			if(sc.WPLx > 1) {
				L.grid = dim3((unsigned)Gm.Ny, (unsigned)(ng * nch * 2));
				L.block = dim3(32 * sc.WPLx);
				L.smem = ((size_t)L.KS * 32 * sc.WPLx * (L.M + 1) + 4 * L.KS * sc.WPLx + 2 * L.KS) * sizeof(cx<R>);
				L.tout = tout;
				launch(wood ? "wood_solve_x" : "expl_solve_x", bytes, [&] {
					if(!launch_solve_xw<R>(L, Gm, slot0, nch, C, fx_cur, sc.plane_x, lx_cur, src, dst, acc_in, acc_out, acc_in2))
						throw BackendError(E_INTERNAL, "no x-solve instance");
				});
				return;
			}
			if(sc.xs) {
				L.grid = dim3((unsigned)((Gm.Ny + LT - 1) / LT), (unsigned)(ng * nch * 2));
				L.block = dim3(32 * LT);
				L.smem = (size_t)LT * L.KS * 32 * (L.M + 1) * sizeof(cx<R>);
				launch(wood ? "wood_solve_x" : "expl_solve_x", bytes, [&] {
					if(!launch_solve_xs<R>(L, Gm, slot0, nch, C, fx_cur, sc.plane_x, lx_cur, src, dst, acc_in, acc_out))
						throw BackendError(E_INTERNAL, "no x-solve instance");
				});
				return;
			}
			L.grid = dim3((unsigned)((Gm.Ny + LT - 1) / LT), (unsigned)(ng * nch * 2));
			L.block = dim3(32 * LT);
			L.smem = (size_t)LT * L.KS * 32 * (L.M + 1) * sizeof(cx<R>);
			L.tout = tout;
			launch(wood ? "wood_solve_x" : "expl_solve_x", bytes, [&] {
				if(!launch_solve_xc<R>(L, Gm, slot0, nch, C, fx_cur, sc.plane_x, lx_cur, src,
						dst, acc_in, acc_out, acc_in2))
					throw BackendError(E_INTERNAL, "no x-solve instance");
			});
		}
		else if(sc.Mxt && sc.WPLt > 1) {
			// long y-lines as several-warps-per-line x-lines of the transposed frame
			const Geom Gt = transposed(Gm);
			L.M = sc.Mxt; L.KS = sc.KSy; L.kind = wood ? ST_WOOD_X : ST_EXPL_Y;
			const int nch = h.spg / L.KS;
			L.grid = dim3((unsigned)Gt.Ny, (unsigned)(ng * nch * 2));
			L.block = dim3(32 * sc.WPLt);
			L.smem = ((size_t)L.KS * 32 * sc.WPLt * (L.M + 1) + 4 * L.KS * sc.WPLt + 2 * L.KS) * sizeof(cx<R>);
			L.tout = tout;
			launch(wood ? "wood_solve_y" : "expl_solve_y", bytes, [&] {
				if(!launch_solve_xw<R>(L, Gt, slot0, nch, ct_cur, fy_cur, sc.plane_y, ly_cur, src, dst, acc_in, acc_out, acc_in2))
					throw BackendError(E_INTERNAL, "no y-solve instance");
			});
		}
		else if(sc.Mxt) {
			// y-lines as x-lines of the transposed frame (fields, coefficients and factors there)
			const Geom Gt = transposed(Gm);
			const int LT = 4;
			L.M = sc.Mxt; L.KS = sc.KSy; L.kind = wood ? ST_WOOD_X : ST_EXPL_Y;
			const int nch = h.spg / L.KS;
			L.grid = dim3((unsigned)((Gt.Ny + LT - 1) / LT), (unsigned)(ng * nch * 2));
			L.block = dim3(32 * LT);
			L.smem = (size_t)LT * L.KS * 32 * (L.M + 1) * sizeof(cx<R>);
			L.tout = tout;
			launch(wood ? "wood_solve_y" : "expl_solve_y", bytes, [&] {
				if(!launch_solve_xc<R>(L, Gt, slot0, nch, ct_cur, fy_cur, sc.plane_y, ly_cur, src, dst, acc_in, acc_out,
						acc_in2))
					throw BackendError(E_INTERNAL, "no y-solve instance");
			});
		}
		else if(sc.Mt) {
			const int LT = 4;
			L.M = sc.Mt; L.KS = sc.KSy; L.kind = wood ? ST_WOOD_Y : ST_EXPL_X;
			const int nch = h.spg / L.KS;
			L.block = dim3(32 * LT);
			L.grid = dim3((unsigned)((Gm.Nx + LT - 1) / LT), (unsigned)(ng * nch * 2));
			L.smem = (size_t)LT * L.KS * 32 * (L.M + 1) * sizeof(cx<R>);
			launch(wood ? "wood_solve_y" : "expl_solve_y", bytes, [&] {
				if(!launch_solve_yt<R>(L, Gm, nch, C, fy_cur, sc.plane_y, ly_cur, src, dst, acc_in, acc_out, acc_in2))
					throw BackendError(E_INTERNAL, "no y-solve instance");
			});
		}
		else if(sc.yq) {
			L.KS = sc.yq; L.kind = wood ? ST_WOOD_Y : ST_EXPL_X;
			const int nch = h.spg / L.KS;
			L.block = dim3(128);
			L.grid = dim3((unsigned)((Gm.Nx + 127) / 128), (unsigned)(ng * nch));
			L.smem = 0;
			if(!scr || scr == src || scr == acc_in || scr == acc_in2) throw BackendError(E_INTERNAL, "y-solve scratch aliases an input");
			launch(wood ? "wood_solve_y" : "expl_solve_y", bytes, [&] {
				if(!launch_solve_yq<R>(L, Gm, nch, C, fy_cur, sc.plane_y, ly_cur, src, scr, dst, acc_in, acc_out, acc_in2))
					throw BackendError(E_INTERNAL, "no y-solve instance");
			});
		}
		else {
			if(sc.ys) {
				const int WS = 8;
				L.M = 0; L.KS = sc.KSy; L.kind = wood ? ST_WOOD_Y : ST_EXPL_X;
				int nch = h.spg / L.KS;
				L.grid = dim3((unsigned)((Gm.Nx + 31) / 32), (unsigned)(ng * nch * 2));
				L.block = dim3(32, WS);
				L.smem = (size_t)(4 * L.KS * WS * 32 + 2 * L.KS * 32) * sizeof(cx<R>);
				launch(wood ? "wood_solve_y" : "expl_solve_y", bytes + fp * 2, [&] {
					if(!launch_solve_ys<R>(L, Gm, slot0, nch, C, fy_cur, sc.plane_y, ly_cur, src, dst, acc_in, acc_out,
							W->T3.as<cx<R>>()))
						throw BackendError(E_INTERNAL, "no y-solve instance");
				});
				return;
			}
			L.M = sc.My; L.KS = sc.KSy; L.kind = wood ? ST_WOOD_Y : ST_EXPL_X;
			int WY = sc.WY;
			if(wood && sc.y1024w) {
				L.M = 8; L.KS = 2;
				WY = (Gm.Ny - 1 + 7) / 8;
			}
			int nch = h.spg / L.KS;
			L.grid = dim3((unsigned)((Gm.Nx + 31) / 32), (unsigned)(ng * nch * 2));
			L.block = dim3(32, WY);
			L.smem = (size_t)((4 + 3 * L.KS) * WY * 32 + L.KS * 32) * sizeof(cx<R>);
			if(yc_values_in_smem(L.M, L.KS, WY > 16 ? 1024 : 512, (int)sizeof(cx<R>)))
				L.smem += (size_t)L.KS * L.M * WY * 32 * sizeof(cx<R>);  // chunk values
			launch(wood ? "wood_solve_y" : "expl_solve_y", bytes, [&] {
				if(!launch_solve_yc<R>(L, Gm, slot0, nch, C, fy_cur, sc.plane_y, ly_cur, src,
						dst, acc_in, acc_out, acc_in2))
					throw BackendError(E_INTERNAL, "no y-solve instance");
			});
		}
	}

	// ParaxialPrimaryEvolutionOperator::apply (ParaxialPrimaryEvolutionOperator.cpp:153-209).
	// only_dirn >= 0: that direction's solves alone (the tuner's timing runs).
	void rec_adi(SampleHost& h, const Geom& Gm, int slot0, int nsl, int ng, int Nw, const cx<R>* C, cx<R>* Fp,
			cx<R>* Tb, cx<R>* T2b, const cx<R>* xsrc, int only_dirn = -1) {
		const int N = Gm.N;
		const double sc = sizeof(cx<R>);
		dim3 gr = pgrid(N, nsl);
		const double fp = (double)N * nsl;
		const SolveCfg& cfg = scfg[h.index];
		for(int dirn = 0; dirn < 2; dirn++) {
			if(only_dirn >= 0 && dirn != only_dirn) continue;
			bool fused = dirn == 0 ? cfg.Mx > 0 : (cfg.My > 0 || cfg.ys || cfg.yq > 0 || cfg.Mt > 0 || cfg.Mxt > 0);
			if(fused) {
				// t0 = solve(f + mu R f) written to T; Woodbury: t_k = solve(mu R' t_{k-1}),
				// F = t0 + t1 + ... accumulated by the solves (the last t_k is not stored).
				rec_solve_fused(dirn, false, h, Gm, slot0, nsl, ng, C, dirn == 0 ? xsrc : Fp, Tb, nullptr, nullptr, nullptr, Tb);
			}
			else {
				if(dirn == 0)
					launch("expl_y", fp * 4 * sc + (double)N * ng * 20 * sc, [&] {
						k_stencil<R, ST_EXPL_Y><<<gr, 256, 0, cs>>>(Gm, slot0, C, Fp, T2b);
					});
				else
					launch("expl_x", fp * 4 * sc + (double)N * ng * 20 * sc, [&] {
						k_stencil<R, ST_EXPL_X><<<gr, 256, 0, cs>>>(Gm, slot0, C, Fp, T2b);
					});
				rec_solve_seq(dirn, h, Gm, slot0, nsl, ng, T2b, Tb, nullptr, nullptr);
			}
			cx<R>* cur = Tb;
			cx<R>* oth = T2b;
			if(Nw == 0) {
				size_t n = (size_t)nsl * 2 * N;
				launch("copy_fields", 2.0 * n * sc, [&] {
					k_copy<R><<<(unsigned)((n + 255) / 256), 256, 0, cs>>>(n, Tb, Fp);
				});
			}
			// Two Woodbury iterates with k_solve_xc / k_solve_yc: the first writes t1 only and the
			// second forms F = (t0 + t1) + t2, the same sums in the same order as accumulating after
			// each iterate, without the first pass over F.
			const bool acc2 = fused && Nw == 2 && solve_takes_acc2(cfg, dirn);
			for(int it = 1; it <= Nw; it++) {
				const cx<R>* ai = it == 1 ? Tb : Fp;
				if(acc2) {
					if(it == 1) rec_solve_fused(dirn, true, h, Gm, slot0, nsl, ng, C, cur, oth, nullptr, nullptr, nullptr, oth);
					// with the transposed-frame y solves, each direction's last solve hands F over
					// transposed (x frame -> transposed frame -> x frame)
					else rec_solve_fused(dirn, true, h, Gm, slot0, nsl, ng, C, cur, nullptr, Tb, Fp, cur, Fp, cfg.Mxt > 0);
				}
				else if(fused) {
					// oth holds t_{it-2} (or nothing), no longer needed: free for the forward values
					rec_solve_fused(dirn, true, h, Gm, slot0, nsl, ng, C, cur, it == Nw ? nullptr : oth, ai, Fp, nullptr, oth);
				}
				else {
					if(dirn == 0)
						launch("wood_x", fp * 4 * sc + (double)N * ng * 14 * sc, [&] {
							k_stencil<R, ST_WOOD_X><<<gr, 256, 0, cs>>>(Gm, slot0, C, cur, oth);
						});
					else
						launch("wood_y", fp * 4 * sc + (double)N * ng * 14 * sc, [&] {
							k_stencil<R, ST_WOOD_Y><<<gr, 256, 0, cs>>>(Gm, slot0, C, cur, oth);
						});
					rec_solve_seq(dirn, h, Gm, slot0, nsl, ng, oth, oth, ai, Fp);
				}
				std::swap(cur, oth);
			}
		}
	}

	// One eager execution with events around every launch; per-kernel totals.
	void profile(std::vector<std::string>& names, std::vector<double>& ms, std::vector<int>& cnt,
			std::vector<double>& bytes) override {
		CK(cudaSetDevice(opt.device));
		profiling = true;
		prof.clear();
		evnext = 0;
		try { record(); }
		catch(...) { profiling = false; throw; }
		profiling = false;
		CK(cudaDeviceSynchronize());
		for(auto& r : prof) {
			float t = 0;
			CK(cudaEventElapsedTime(&t, r.a, r.b));
			size_t k = 0;
			for(; k < names.size(); k++) if(names[k] == r.name) break;
			if(k == names.size()) { names.push_back(r.name); ms.push_back(0); cnt.push_back(0); bytes.push_back(0); }
			ms[k] += t;
			cnt[k] += 1;
			bytes[k] += r.bytes;
		}
	}

	void execute(nbpm_timing* tm) override {
		CK(cudaSetDevice(opt.device));
		if(opt.use_graph) {
			if(!gexec) {
				cudaGraph_t graph;
				CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
				try { record(); }
				catch(...) {
					cudaStreamEndCapture(stream, &graph);
					if(graph) cudaGraphDestroy(graph);
					throw;
				}
				CK(cudaStreamEndCapture(stream, &graph));
				CK(cudaGraphInstantiate(&gexec, graph, 0));
				cudaGraphDestroy(graph);
			}
			CK(cudaEventRecord(ev[0], stream));
			CK(cudaGraphLaunch(gexec, stream));
			CK(cudaEventRecord(ev[1], stream));
		}
		else {
			CK(cudaEventRecord(ev[0], stream));
			record();
			CK(cudaEventRecord(ev[1], stream));
		}
		CK(cudaStreamSynchronize(stream));
		CK(cudaGetLastError());
		float ms = 0;
		CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
		last_slab_ms = 0;
		if(tm) {
			tm->compute_ms = ms;
			tm->kernel_launches = launches;
			long long vs = 0;
			for(auto& hp : S) vs += (long long)hp->geom.N * (hp->geom.Nz - 1) * hp->slots;
			tm->voxel_steps = vs;
		}
	}

	long long device_bytes() const override { return dev_bytes; }
	double slab_ms() const override { return last_slab_ms; }
	int slabs() const override { return S.empty() ? 0 : S[0]->geom.Nz - 1; }
	long long voxel_steps() const override {
		long long vs = 0;
		for(auto& hp : S) vs += (long long)hp->geom.N * (hp->geom.Nz - 1) * hp->slots;
		return vs;
	}

	PassState sps;
	cudaEvent_t eDone = nullptr;
	void step_begin() override {
		if(S.size() != 1 || gpp(*S[0]) != S[0]->G) throw BackendError(E_ARG, "stepped plans hold one sample in one pass");
		CK(cudaSetDevice(opt.device));
		if(!eDone) CK(cudaEventCreateWithFlags(&eDone, cudaEventDisableTiming));
		select(*S[0]);
		rec_prologue(*S[0]);
		sps = rec_pass_begin(*S[0], 0);
		rec_bulk(*S[0], sps, 0, nullptr);
	}
	int step_advance(int nslabs) override {
		CK(cudaSetDevice(opt.device));
		select(*S[0]);
		SampleHost& h = *S[0];
		int end = std::min(h.geom.Nz - 1, sps.iz + std::max(0, nslabs));
		rec_pass_slabs(h, sps, end);
		return h.geom.Nz - 1 - sps.iz;
	}
	void step_finish() override {
		CK(cudaSetDevice(opt.device));
		select(*S[0]);
		SampleHost& h = *S[0];
		rec_pass_end(h, sps);
		rec_screen(h);
		size_t n = (size_t)h.slots * 2 * h.geom.N;
		if(sizeof(R) == sizeof(double)) {
			CK(cudaMemcpyAsync(h.E, h.F.p, n * sizeof(cx<double>), cudaMemcpyDeviceToHost, stream));
		}
		else {
			k_widen<R><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, h.F.as<cx<R>>(), W->stage.as<cx<double>>());
			CK(cudaGetLastError());
			CK(cudaMemcpyAsync(h.E, W->stage.p, n * sizeof(cx<double>), cudaMemcpyDeviceToHost, stream));
		}
		CK(cudaEventRecord(eDone, stream));
	}
	void sync() override {
		for(auto& hp : S) {
			CK(cudaStreamSynchronize(hp->lane.main));
			CK(cudaStreamSynchronize(hp->lane.setup));
		}
	}
	bool step_done() override {
		cudaError_t e = cudaEventQuery(eDone);
		if(e == cudaErrorNotReady) return false;
		CK(e);
		return true;
	}

	bool solve_config(int sample, std::string& cfg, std::string& note) const override {
		if(sample < 0 || sample >= (int)S.size() || sample >= (int)scfg.size()) return false;
		cfg = scfg[sample].str();
		note = sample < (int)tune_notes.size() ? tune_notes[sample] : std::string();
		return true;
	}

	bool fields_view(int sample, PlanFieldsView& v) const override {
		if(sample < 0 || sample >= (int)S.size()) return false;
		const SampleHost& h = *S[sample];
		v.ptr = h.F.p;
		v.n = (size_t)h.slots * 2 * h.geom.N;
		v.fp32 = sizeof(R) == sizeof(float);
		v.Nx = h.s.Nx;
		v.Ny = h.s.Ny;
		v.Nl = (int)h.s.wavelengths.size();
		v.Nq = (int)h.s.q.size();
		v.device = opt.device;
		v.stream = stream;
		return true;
	}
};

}  // namespace nbpm

using namespace nbpm;

struct nbpm_plan {
	std::unique_ptr<PlanBase> impl;
};

std::unique_ptr<PlanBase> nbpm::make_plan_host(int n_samples, const nbpm_sample* samples, const nbpm_options& o) {
	if(n_samples <= 0 || !samples) throw BackendError(E_ARG, "invalid plan arguments");
	if(o.precision == NBPM_FP64) {
		std::unique_ptr<Plan<double>> p(new Plan<double>(o));
		p->setup_host(n_samples, samples);
		return std::unique_ptr<PlanBase>(p.release());
	}
	if(o.precision == NBPM_FP32) {
		std::unique_ptr<Plan<float>> p(new Plan<float>(o));
		p->setup_host(n_samples, samples);
		return std::unique_ptr<PlanBase>(p.release());
	}
	throw BackendError(E_ARG, "unknown precision");
}

bool nbpm::plan_fields_view(nbpm_plan* p, int sample, PlanFieldsView& v) {
	return p && p->impl && p->impl->fields_view(sample, v);
}

static int fail(int code, const std::string& msg) {
	g_last_error = msg;
	return code;
}

#define API_GUARD(...)                                                         \
	try { __VA_ARGS__ }                                                                 \
	catch(BackendError& e) { return fail(e.code, e.what()); }                    \
	catch(std::bad_alloc&) { return fail(E_MEMORY, "host out of memory"); }      \
	catch(std::exception& e) { return fail(E_INTERNAL, e.what()); }              \
	catch(...) { return fail(E_INTERNAL, "unknown exception"); }

extern "C" {

void nbpm_default_options(nbpm_options* o) {
	if(!o) return;
	o->precision = NBPM_FP64;
	o->groups_per_pass = 0;
	o->use_graph = 1;
	o->device = 0;
	o->verbose = 0;
	o->tune = 1;
	o->solve_config = nullptr;
}

const char* nbpm_last_error(void) { return g_last_error.c_str(); }

int nbpm_eval_index(const char* expr, double lambda, double* out) {
	g_last_error.clear();
	API_GUARD({
		if(!expr || !out) return fail(E_ARG, "null argument");
		*out = eval_index(expr, lambda, "expression");
		return 0;
	})
}

int nbpm_mask_weights(const char* json_str, const char* mask_formula, const double* mask_vals, int n_mask_vals,
		unsigned char* mask_out, double* weights_out) {
	g_last_error.clear();
	API_GUARD({
		if(!json_str || !mask_vals || !mask_out || !weights_out) return fail(E_ARG, "null argument");
		BackendSettings s = parse_settings(json_str);
		size_t nv = (size_t)s.Nx * s.Ny * s.Nz;
		if((size_t)n_mask_vals != nv) return fail(E_SIZE, "Wrong dimension for the mask pointer array");
		std::vector<unsigned char> m;
		std::vector<double> w;
		mask_weights(s, mask_vals, mask_formula ? mask_formula : "", m, w);
		std::memcpy(mask_out, m.data(), m.size());
		if(!w.empty()) std::memcpy(weights_out, w.data(), w.size() * sizeof(double));
		return 0;
	})
}
const char* nbpm_version(void) { return "nbpm 0.1.0 (sm_103a)"; }

int nbpm_plan_create(int n_samples, const nbpm_sample* samples, const nbpm_options* opts, nbpm_plan** out) {
	g_last_error.clear();
	API_GUARD({
		if(!out || n_samples <= 0 || !samples) return fail(E_ARG, "invalid plan arguments");
		*out = nullptr;
		nbpm_options o;
		nbpm_default_options(&o);
		if(opts) o = *opts;
		if(o.precision != NBPM_FP64 && o.precision != NBPM_FP32) return fail(E_ARG, "unknown precision");
		std::unique_ptr<nbpm_plan> p(new nbpm_plan());
		if(o.precision == NBPM_FP64) {
			auto* pl = new Plan<double>(o);
			p->impl.reset(pl);
			pl->setup(n_samples, samples);
		}
		else {
			auto* pl = new Plan<float>(o);
			p->impl.reset(pl);
			pl->setup(n_samples, samples);
		}
		*out = p.release();
		return 0;
	})
}

int nbpm_plan_upload(nbpm_plan* p) {
	API_GUARD({
		if(!p) return fail(E_ARG, "null plan");
		p->impl->upload();
		return 0;
	})
}

int nbpm_plan_execute(nbpm_plan* p, nbpm_timing* t) {
	API_GUARD({
		if(!p) return fail(E_ARG, "null plan");
		p->impl->execute(t);
		return 0;
	})
}

int nbpm_plan_download(nbpm_plan* p) {
	API_GUARD({
		if(!p) return fail(E_ARG, "null plan");
		p->impl->download();
		return 0;
	})
}

int nbpm_plan_slab_ms(nbpm_plan* p, double* ms) {
	if(!p || !ms) return fail(E_ARG, "null argument");
	*ms = p->impl->slab_ms();
	return 0;
}

int nbpm_plan_profile(nbpm_plan* p, char (*names)[48], double* ms, int* launches, double* bytes, int* n) {
	API_GUARD({
		if(!p || !names || !ms || !launches || !bytes || !n) return fail(E_ARG, "null argument");
		std::vector<std::string> nm;
		std::vector<double> t, b;
		std::vector<int> c;
		p->impl->profile(nm, t, c, b);
		int k = std::min<int>(*n, (int)nm.size());
		for(int i = 0; i < k; i++) {
			std::snprintf(names[i], 48, "%s", nm[i].c_str());
			ms[i] = t[i];
			launches[i] = c[i];
			bytes[i] = b[i];
		}
		*n = k;
		return 0;
	})
}

long long nbpm_plan_device_bytes(const nbpm_plan* p) { return p ? p->impl->device_bytes() : 0; }

static void copy_out(const std::string& src, char* dst, int n) {
	if(!dst || n <= 0) return;
	std::snprintf(dst, (size_t)n, "%s", src.c_str());
}

int nbpm_plan_solve_config(const nbpm_plan* p, int sample, char* config, int n_config, char* report, int n_report) {
	API_GUARD({
		if(!p || !config || n_config <= 0) return fail(E_ARG, "null argument");
		std::string c, note;
		if(!p->impl->solve_config(sample, c, note)) return fail(E_ARG, "sample index out of range");
		copy_out(c, config, n_config);
		copy_out(note, report, n_report);
		return 0;
	})
}

int nbpm_solve_candidates(const char* json_str, int precision, int groups_per_pass, char* out, int n) {
	g_last_error.clear();
	API_GUARD({
		if(!json_str || !out || n <= 0) return fail(E_ARG, "null argument");
		if(precision != NBPM_FP64 && precision != NBPM_FP32) return fail(E_ARG, "unknown precision");
		BackendSettings s = parse_settings(json_str);
		SolveShape sh;
		sh.Nx = s.Nx; sh.Ny = s.Ny; sh.spg = 2 * (int)s.q.size(); sh.nw = s.n_woodbury;
		int G = (int)s.wavelengths.size();
		sh.ng = groups_per_pass <= 0 ? G : std::max(1, std::min(groups_per_pass, G));
		sh.fp32 = precision == NBPM_FP32;
		int dev = 0, v = 0;
		if(cudaGetDevice(&dev) == cudaSuccess) {
			if(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0) sh.nsm = v;
			if(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess && v > 0) sh.smem = (size_t)v;
		}
		cudaGetLastError();
		std::string r = "x=";
		auto xs = x_candidates(sh), ys = y_candidates(sh);
		for(size_t i = 0; i < xs.size(); i++) r += (i ? "|" : "") + xs[i].xstr();
		r += "\ny=";
		for(size_t i = 0; i < ys.size(); i++) r += (i ? "|" : "") + ys[i].ystr();
		r += "\ndefault=" + heuristic(sh).str();
		if((int)r.size() >= n) return fail(E_SIZE, "output buffer too small");
		copy_out(r, out, n);
		return 0;
	})
}

int nbpm_tune_cache_clear(void) {
	tune_cache_clear();
	return 0;
}

int nbpm_plan_destroy(nbpm_plan* p) {
	delete p;
	return 0;
}

}  // extern "C"

namespace {
// One kept plan: a call with the same settings, sizes and options as the previous one (no mask,
// no bulk output) reuses its device buffers and recorded graph; only the inputs are uploaded
// again. NBPM_PLAN_CACHE=0 disables it; nbpm_release_plan_cache frees it.
struct PlanCache {
	std::mutex m;
	std::string key;
	std::unique_ptr<nbpm_plan> plan;
};
// never destroyed: a kept plan is released with the process, not by a static destructor that
// could run after the CUDA runtime has shut down
PlanCache& plan_cache() {
	static PlanCache* c = new PlanCache();
	return *c;
}

std::string plan_key(int n, const nbpm_sample* s, const nbpm_options* opts) {
	nbpm_options o;
	nbpm_default_options(&o);
	if(opts) o = *opts;
	std::string k = std::to_string(o.precision) + "/" + std::to_string(o.groups_per_pass) + "/" +
		std::to_string(o.use_graph) + "/" + std::to_string(o.device) + "/" + std::to_string(o.verbose) + "/" +
		std::to_string(o.tune) + "/" + (o.solve_config ? o.solve_config : "");
	for(int i = 0; i < n; i++) {
		if(!s[i].json_str) return std::string();
		k += "|" + std::to_string(s[i].n_lc_vals) + "/" + std::to_string(s[i].n_E_vals) + "/" +
			std::to_string(s[i].mask_vals ? s[i].n_mask_vals : -1) + "/" + (s[i].mask_formula ? s[i].mask_formula : "") +
			"/" + s[i].json_str;
	}
	return k;
}

bool plan_cache_on() {
	const char* e = std::getenv("NBPM_PLAN_CACHE");
	return !(e && std::atoi(e) == 0);
}

// Upload, execute, download of one plan with the timing breakdown.
static int run_plan_once(nbpm_plan* p, nbpm_timing* timing) {
	API_GUARD({
		auto t0 = std::chrono::steady_clock::now();
		p->impl->upload();
		auto t1 = std::chrono::steady_clock::now();
		nbpm_timing tm{};
		p->impl->execute(&tm);
		auto t2 = std::chrono::steady_clock::now();
		p->impl->download();
		auto t3 = std::chrono::steady_clock::now();
		if(timing) {
			*timing = tm;
			timing->upload_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
			timing->download_ms = std::chrono::duration<double, std::milli>(t3 - t2).count();
			timing->total_ms = std::chrono::duration<double, std::milli>(t3 - t0).count();
		}
		return 0;
	})
}
}  // namespace

extern "C" {

int nbpm_release_plan_cache(void) {
	std::lock_guard<std::mutex> lk(plan_cache().m);
	plan_cache().plan.reset();
	plan_cache().key.clear();
	return 0;
}

int nbpm_run_batch(int n_samples, const nbpm_sample* samples, const nbpm_options* opts, nbpm_timing* timing) {
	g_last_error.clear();
	if(n_samples <= 0 || !samples) return fail(E_ARG, "invalid plan arguments");
	// the kept plan, if this call matches it and no other call holds it
	std::unique_lock<std::mutex> lk(plan_cache().m, std::defer_lock);
	const std::string key = plan_cache_on() ? plan_key(n_samples, samples, opts) : std::string();
	if(!key.empty()) (void)lk.try_lock();
	nbpm_plan* p = nullptr;
	std::unique_ptr<nbpm_plan> guard;
	bool reused = false;
	if(lk.owns_lock() && plan_cache().plan && plan_cache().key == key) {
		p = plan_cache().plan.get();
		int rc = [&]() -> int { API_GUARD({ return p->impl->rebind(n_samples, samples) ? 0 : -1; }) }();
		if(rc > 0) { plan_cache().plan.reset(); plan_cache().key.clear(); return rc; }
		reused = rc == 0;
	}
	if(!reused) {
		if(lk.owns_lock()) { plan_cache().plan.reset(); plan_cache().key.clear(); }
		int rc = nbpm_plan_create(n_samples, samples, opts, &p);
		if(rc) return rc;
		guard.reset(p);
	}
	int rc = run_plan_once(p, timing);
	if(rc) {
		if(!guard) { plan_cache().plan.reset(); plan_cache().key.clear(); }
		return rc;
	}
	if(guard && lk.owns_lock() && p->impl->reusable()) {
		plan_cache().plan = std::move(guard);
		plan_cache().key = key;
	}
	return 0;
}

int nbpm_run_backend_ex(const char* json_str, const char* mask_formula, const double* lc_field_vals,
		int n_lc_vals, const double* mask_vals, int n_mask_vals, double* E_field_vals, int n_E_vals,
		const nbpm_options* opts, nbpm_timing* timing) {
	nbpm_sample s;
	s.json_str = json_str;
	s.mask_formula = mask_formula;
	s.lc_field_vals = lc_field_vals;
	s.n_lc_vals = n_lc_vals;
	s.mask_vals = mask_vals;
	s.n_mask_vals = n_mask_vals;
	s.E_field_vals = E_field_vals;
	s.n_E_vals = n_E_vals;
	return nbpm_run_batch(1, &s, opts, timing);
}

int nbpm_run_backend_without_mask(const char* json_str, const double* lc_field_vals, int n_lc_vals,
		double* E_field_vals, int n_E_vals) {
	return nbpm_run_backend_ex(json_str, nullptr, lc_field_vals, n_lc_vals, nullptr, 0, E_field_vals, n_E_vals,
		nullptr, nullptr);
}

int nbpm_run_backend_with_mask(const char* json_str, const char* mask_formula, const double* lc_field_vals,
		int n_lc_vals, const double* mask_vals, int n_mask_vals, double* E_field_vals, int n_E_vals) {
	return nbpm_run_backend_ex(json_str, mask_formula ? mask_formula : "", lc_field_vals, n_lc_vals,
		mask_vals, n_mask_vals, E_field_vals, n_E_vals, nullptr, nullptr);
}

}  // extern "C"
