// Microscope stage after the backend, on the device and in FP64: objective focalisation of
// the output fields and the incoherent (Koehler) spectrum sum that a micrograph is made from.
//
// OpticalFields (HighLevelPythonInterface/nemaktis/light_propagator.py):
//   wavevector grid :576-596, spacings :599, objective filter and NA mask :614-646,
//   update_NA_objective :702-705, focus_fields :708-719.
// FieldViewer (nemaktis/field_viewer.py):
//   _update_specter :348-388, _update_averaged_specter :391-455, Jones matrices :472-513,
//   q_int_func / get_q_idx :515-518.
//
// Device data per microscope (all FP64):
//   vals      (Nl, Nq, 4, Ny, Nx) complex  input fields (reference layout)
//   focused   (Nl, Nq, 4, Ny, Nx) complex  focused fields
//   tab       (Nl, Nq, Ny, Nx) {theta, |k+p|^2}: theta = Arg of the objective filter
//             exp(i(sqrt(kn^2 - |k+p|^2) - kn)) where |k+p|^2 < kn^2, NaN outside
//   filt      (Nl, Nq, Ny, Nx) complex  mask * filter^|zf| / (Nx Ny) for the current focus
//   spectrum  (Ny, Nx, Nl) double
// Focalisation = x-line FFT (vals -> focused), one fused kernel per y-line doing the forward
// FFT, the filter product and the inverse FFT, then the inverse x-line FFT.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/nbpm.h"
#include "cplx.cuh"
#include "fft_kernels.cuh"
#include "plan_iface.h"

namespace nbpm {

void set_last_error(const std::string& m);

namespace {

struct MsError {
	int code;
	std::string msg;
};

#define MCK(call)                                                                                    \
	do {                                                                                             \
		cudaError_t e_ = (call);                                                                     \
		if(e_ != cudaSuccess)                                                                        \
			throw MsError{e_ == cudaErrorMemoryAllocation ? NBPM_ERR_MEMORY : NBPM_ERR_CUDA,         \
				std::string(cudaGetErrorString(e_)) + " at " + #call};                                \
	} while(0)

struct Buf {
	void* p = nullptr;
	Buf() = default;
	Buf(const Buf&) = delete;
	Buf& operator=(const Buf&) = delete;
	~Buf() { if(p) cudaFree(p); }
	void alloc(size_t b) {
		if(p) { cudaFree(p); p = nullptr; }
		if(b) MCK(cudaMalloc(&p, b));
	}
	template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

constexpr double PI_NP = 3.141592653589793;  // numpy.pi

// ---------------------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ double norm2(cx<double> a) { return a.x * a.x + a.y * a.y; }

// theta and |k+p|^2 per (l, q, iy, ix), light_propagator.py:621-642. The products and sums
// are rounded one by one (no fused multiply-add) so the comparisons against kn^2 and
// (k0 NA)^2 decide as numpy's do.
__global__ void k_objective_table(int Nx, int Ny, int Nl, int Nq, double dx, double dy,
		const double* __restrict__ wl, const double* __restrict__ nout, const double* __restrict__ qv,
		double2* __restrict__ tab) {
	const long long N = (long long)Nx * Ny;
	long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if(t >= N * Nl * Nq) return;
	int ix = (int)(t % Nx);
	int iy = (int)((t / Nx) % Ny);
	int lq = (int)(t / N);
	int l = lq / Nq, q = lq % Nq;
	double tx = __dsub_rn(fmod(__dadd_rn((double)ix, __dmul_rn(0.5, (double)Nx)), (double)Nx), __dmul_rn(0.5, (double)Nx));
	double ty = __dsub_rn(fmod(__dadd_rn((double)iy, __dmul_rn(0.5, (double)Ny)), (double)Ny), __dmul_rn(0.5, (double)Ny));
	double kx = __ddiv_rn(__dmul_rn(__dmul_rn(tx, 2.0), PI_NP), __dmul_rn((double)Nx, dx));
	double ky = __ddiv_rn(__dmul_rn(__dmul_rn(ty, 2.0), PI_NP), __dmul_rn((double)Ny, dy));
	double k0 = __ddiv_rn(2.0 * PI_NP, wl[l]);
	double kn = __ddiv_rn(__dmul_rn(2.0 * PI_NP, nout[l]), wl[l]);
	double px = __dmul_rn(k0, qv[2 * q]), py = __dmul_rn(k0, qv[2 * q + 1]);
	double ax = __dadd_rn(kx, px), ay = __dadd_rn(ky, py);
	double ksq = __dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay));
	double kn2 = __dmul_rn(kn, kn);
	double theta = nan("");
	if(ksq < kn2) {
		double ph = __dsub_rn(__dsqrt_rn(__dsub_rn(kn2, ksq)), kn);
		double s, c;
		sincos(ph, &s, &c);
		theta = atan2(s, c);
	}
	tab[t] = make_double2(theta, ksq);
}

// mask * filter^|zf| (conjugated for zf < 0) times 1/(Nx Ny), light_propagator.py:702-719.
// The power is the principal-branch one of numpy: exp(a * i * theta), 0^0 = 1.
__global__ void k_focus_filter(long long N, int Nl, int Nq, double NA, double a, int conj_f, double scale,
		const double* __restrict__ wl, const double2* __restrict__ tab, cx<double>* __restrict__ filt) {
	long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if(t >= N * Nl * Nq) return;
	int l = (int)(t / (N * Nq));
	double k0 = __ddiv_rn(2.0 * PI_NP, wl[l]);
	double kna = __dmul_rn(k0, NA);
	double2 e = tab[t];
	cx<double> f = mk(0.0, 0.0);
	if(e.y < __dmul_rn(kna, kna)) {
		if(a == 0.0) f = mk(1.0, 0.0);
		else if(!isnan(e.x)) {
			double s, c;
			sincos(a * e.x, &s, &c);
			f = mk(c, s);
		}
	}
	if(conj_f) f.y = -f.y;
	filt[t] = f * scale;
}

// One block transforms `lpb` y-lines (adjacent columns x of one plane (l, q, comp)): forward
// FFT, product with the focus filter of (l, q), inverse FFT (unscaled; the scale is in filt).
__global__ void k_focus_cols(cx<double>* F, FftPlan1D P, int nlines, int Nx, long long N, int lpb,
		const cx<double>* __restrict__ tw, const cx<double>* __restrict__ filt) {
	extern __shared__ unsigned char smem_raw[];
	cx<double>* sA = reinterpret_cast<cx<double>*>(smem_raw);
	const int n = P.n, pitch = n + 1;
	cx<double>* sB = sA + (size_t)lpb * pitch;
	int l0 = blockIdx.x * lpb;
	int nl = min(lpb, nlines - l0);
	if(nl <= 0) return;
	auto addr = [&](int line, int i) {
		return (long long)(line / Nx) * N + (long long)i * Nx + (line % Nx);
	};
	const int tot = nl * n;
	for(int e = threadIdx.x; e < tot; e += blockDim.x) {
		int li = e % nl, i = e / nl;
		sA[li * pitch + i] = F[addr(l0 + li, i)];
	}
	__syncthreads();
	cx<double>* res = fft_stages<double>(sA, sB, P, nl, tw, -1);
	for(int e = threadIdx.x; e < tot; e += blockDim.x) {
		int li = e % nl, i = e / nl;
		int line = l0 + li;
		long long lq = (line / Nx) / 4;  // plane = (l*Nq + q)*4 + comp
		res[li * pitch + i] = res[li * pitch + i] * filt[lq * N + (long long)i * Nx + (line % Nx)];
	}
	__syncthreads();
	cx<double>* res2 = fft_stages<double>(res, res == sA ? sB : sA, P, nl, tw, +1);
	for(int e = threadIdx.x; e < tot; e += blockDim.x) {
		int li = e % nl, i = e / nl;
		F[addr(l0 + li, i)] = res2[li * pitch + i];
	}
}

// Spectrum per (pixel, l): sum_k w[k] * 0.5 * || post_l . T . pre_l ||_F^2 over the
// wavevectors q = q_start + k, with T[j][i] = fields[l, q, 2i+j] (field_viewer.py:348-455).
// pre/post hold 4 complex values per wavelength (row-major 2x2). plain: both are identities.
__global__ void k_spectrum(const cx<double>* __restrict__ F, long long N, int Nl, int Nq, int q_start, int nw,
		const double* __restrict__ w, const cx<double>* __restrict__ pre, const cx<double>* __restrict__ post,
		int plain, double* __restrict__ out) {
	long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	int l = blockIdx.y;
	if(p >= N) return;
	cx<double> A[4], B[4];
	for(int i = 0; i < 4; i++) { A[i] = pre[4 * l + i]; B[i] = post[4 * l + i]; }
	double acc = 0;
	for(int k = 0; k < nw; k++) {
		const cx<double>* f = F + ((long long)(l * Nq + q_start + k) * 4) * N + p;
		cx<double> v0 = f[0], v1 = f[N], v2 = f[2 * N], v3 = f[3 * N];
		double s;
		if(plain) s = norm2(v0) + norm2(v1) + norm2(v2) + norm2(v3);
		else {
			// T = [[v0, v2], [v1, v3]]; X = T . pre; Y = post . X
			cx<double> x00 = v0 * A[0] + v2 * A[2], x01 = v0 * A[1] + v2 * A[3];
			cx<double> x10 = v1 * A[0] + v3 * A[2], x11 = v1 * A[1] + v3 * A[3];
			cx<double> y00 = B[0] * x00 + B[1] * x10, y01 = B[0] * x01 + B[1] * x11;
			cx<double> y10 = B[2] * x00 + B[3] * x10, y11 = B[2] * x01 + B[3] * x11;
			s = norm2(y00) + norm2(y01) + norm2(y10) + norm2(y11);
		}
		acc += w[k] * (0.5 * s);
	}
	out[p * Nl + l] = acc;
}

__global__ void k_widen_f32(size_t n, const cx<float>* __restrict__ a, cx<double>* __restrict__ b) {
	size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n) b[i] = mk((double)a[i].x, (double)a[i].y);
}

// ---------------------------------------------------------------------------------------
// Host: Jones matrices and Koehler weights (field_viewer.py:391-455, 472-518), FP64.
// ---------------------------------------------------------------------------------------
using C = std::complex<double>;
struct M2 {
	C a[4];  // row-major
};
static M2 eye() { return M2{{C(1, 0), C(0, 0), C(0, 0), C(1, 0)}}; }
static M2 mul(const M2& x, const M2& y) {
	return M2{{x.a[0] * y.a[0] + x.a[1] * y.a[2], x.a[0] * y.a[1] + x.a[1] * y.a[3],
		x.a[2] * y.a[0] + x.a[3] * y.a[2], x.a[2] * y.a[1] + x.a[3] * y.a[3]}};
}
static M2 polariser(double ang) {
	double c = std::cos(ang * PI_NP / 180), s = std::sin(ang * PI_NP / 180);
	return M2{{C(c * c), C(c * s), C(c * s), C(s * s)}};
}
static M2 waveplate(int kind, double ang, double lambda) {
	double c = std::cos(ang * PI_NP / 180), s = std::sin(ang * PI_NP / 180);
	const C I(0, 1);
	if(kind == NBPM_WAVEPLATE_QUARTER) {
		C ph = std::exp(-I * (PI_NP / 4));
		C o = (C(1) - I) * (c * s);
		return M2{{ph * (c * c + I * (s * s)), ph * o, ph * o, ph * (s * s + I * (c * c))}};
	}
	if(kind == NBPM_WAVEPLATE_HALF) {
		C ph = std::exp(-I * (PI_NP / 2));
		return M2{{ph * (c * c - s * s), ph * (2 * c * s), ph * (2 * c * s), ph * (s * s - c * c)}};
	}
	// tint-sensitive: full wave at 0.540 um
	C g = std::exp(I * (PI_NP * 0.540 / lambda)), gc = std::conj(g);
	C o = (gc - g) * (c * s);
	return M2{{gc * (c * c) + g * (s * s), o, o, gc * (s * s) + g * (c * c)}};
}

static double q_int_func(double q, double qp) { return q - std::atanh(q) - qp * std::log(1 - q * q) / 2; }
static int get_q_idx(int r) { return 1 + 3 * r * (r - 1); }

struct Weights {
	int q_start = 0;
	std::vector<double> w;
};

static Weights koehler_weights(double NA, double max_NA, int Nr, int k1d) {
	Weights W;
	if(NA < 1e-8) {
		W.q_start = k1d ? Nr - 1 : 0;
		W.w.assign(1, 1.0);
		return W;
	}
	double dq = (Nr > 1 && max_NA > 0) ? max_NA / (Nr - 1) : 1.0;
	int rmax = std::min(Nr - 1, (int)std::ceil(NA / dq));
	if(!k1d) {
		std::vector<double>& w = W.w;
		w.assign((size_t)get_q_idx(rmax + 1), 0.0);
		auto put = [&](int a, int b, double v) {  // slice assignment w[a:b] = v
			int n = (int)w.size();
			a = std::min(std::max(a, 0), n);
			b = std::min(std::max(b, 0), n);
			for(int i = a; i < b; i++) w[i] = v;
		};
		if(rmax == 1) {
			w[0] = (q_int_func(NA, dq) - q_int_func(0, dq)) / dq;
			put(1, 7, (q_int_func(0, 0) - q_int_func(NA, 0)) / (6 * dq));
		}
		else {
			w[0] = (q_int_func(dq, dq) - q_int_func(0, dq)) / dq;
			for(int r = 1; r < rmax - 1; r++)
				put(get_q_idx(r), get_q_idx(r + 1),
					(q_int_func((r + 1) * dq, (r + 1) * dq) + q_int_func((r - 1) * dq, (r - 1) * dq)
						- 2 * q_int_func(r * dq, r * dq)) / (6 * r * dq));
			put(get_q_idx(rmax - 1), get_q_idx(rmax),
				(q_int_func(NA, rmax * dq) + q_int_func((rmax - 2) * dq, (rmax - 2) * dq)
					- 2 * q_int_func((rmax - 1) * dq, (rmax - 1) * dq)) / (6 * (rmax - 1) * dq));
			put(get_q_idx(rmax), get_q_idx(rmax + 1),
				(q_int_func((rmax - 1) * dq, (rmax - 1) * dq) - q_int_func(NA, (rmax - 1) * dq)) / (6 * rmax * dq));
		}
		double f = 2 / (NA * NA);
		for(double& x : w) x = x * f;
		return W;
	}
	if(rmax < 1)
		throw MsError{NBPM_ERR_ARG, "Koehler 1-D spectrum needs at least 2 radial wavevectors"};
	double edge = NA - (rmax - 1) * dq;
	std::vector<double>& w = W.w;
	w.assign((size_t)(2 * rmax + 1), dq);
	w[0] = w[w.size() - 1] = edge * edge / (2 * dq);
	if(rmax == 1) w[1] = edge * (2 - edge / dq);
	else w[1] = w[w.size() - 2] = edge * (1 - edge / (2 * dq)) + dq / 2;
	for(double& x : w) x = x / (2 * NA);
	W.q_start = Nr - 1 - rmax;
	return W;
}

}  // namespace

struct Microscope {
	nbpm_microscope_params P{};
	std::vector<double> wl, nout, qv;
	int Nx = 0, Ny = 0, Nl = 0, Nq = 0;
	long long N = 0;
	double dx = 0, dy = 0;
	double NA = 0, z = 0;
	size_t smem_limit = 0;
	cudaStream_t st = nullptr;
	cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
	Buf dwl, dnout, dqv, tab, filt, vals, foc, spec, dw, dpre, dpost, twx, twy;
	size_t nw_cap = 0;
	float focus_ms = 0, spectrum_ms = 0;
	long long bytes = 0;

	~Microscope() {
		if(st) cudaStreamSynchronize(st);
		for(auto& e : ev) if(e) cudaEventDestroy(e);
		if(st) cudaStreamDestroy(st);
	}

	size_t nvals() const { return (size_t)Nl * Nq * 4 * N; }

	void twiddles(Buf& b, int n) {
		std::vector<cx<double>> h(n);
		for(int k = 0; k < n; k++) {
			double a = 2 * PI_NP * (double)k / (double)n;
			h[k] = mk(std::cos(a), -std::sin(a));
		}
		b.alloc(sizeof(cx<double>) * n);
		MCK(cudaMemcpyAsync(b.p, h.data(), sizeof(cx<double>) * n, cudaMemcpyHostToDevice, st));
		MCK(cudaStreamSynchronize(st));
	}

	void setup(const nbpm_microscope_params& in) {
		P = in;
		if(in.Nx < 1 || in.Ny < 1) throw MsError{NBPM_ERR_ARG, "mesh_dimensions must be >= 1"};
		if(in.n_wavelengths < 1 || !in.wavelengths) throw MsError{NBPM_ERR_ARG, "no wavelengths"};
		if(in.N_radial_wavevectors < 1) throw MsError{NBPM_ERR_ARG, "N_radial_wavevectors must be >= 1"};
		Nx = in.Nx; Ny = in.Ny; N = (long long)Nx * Ny; Nl = in.n_wavelengths;
		dx = in.Lx / std::max(1.0, (double)Nx - 1.0);
		dy = in.Ly / std::max(1.0, (double)Ny - 1.0);
		wl.assign(in.wavelengths, in.wavelengths + Nl);
		nout.assign((size_t)Nl, 1.0);
		if(in.n_out) nout.assign(in.n_out, in.n_out + Nl);
		// wavevectors: explicit, else the grid of light_propagator.py:576-596
		if(in.n_wavevectors > 0) {
			if(!in.wavevectors) throw MsError{NBPM_ERR_ARG, "n_wavevectors > 0 but wavevectors is NULL"};
			qv.assign(in.wavevectors, in.wavevectors + 2 * (size_t)in.n_wavevectors);
		}
		else {
			int Nr = in.N_radial_wavevectors;
			double mc = in.max_NA_condenser;
			if(in.koehler_1D && (Nx == 1 || Ny == 1)) {
				int axis = Nx == 1 ? 1 : 0;
				qv.assign(2 * (size_t)(2 * Nr - 1), 0.0);
				for(int ir = 1; ir < Nr; ir++) {
					double b = ir * mc / (Nr - 1);
					qv[2 * (Nr - 1 + ir) + axis] = b;
					qv[2 * (Nr - 1 - ir) + axis] = -b;
				}
			}
			else {
				qv.assign(2 * (size_t)(1 + 3 * Nr * (Nr - 1)), 0.0);
				for(int ir = 1; ir < Nr; ir++) {
					double b = ir * mc / (Nr - 1);
					for(int k = 0; k < 6 * ir; k++) {
						double phi = k * PI_NP / (3 * ir);
						size_t o = 2 * (size_t)(1 + 3 * ir * (ir - 1) + k);
						qv[o] = b * std::cos(phi);
						qv[o + 1] = b * std::sin(phi);
					}
				}
			}
		}
		Nq = (int)(qv.size() / 2);
		NA = in.max_NA_objective;
		FftPlan1D px, py;
		if(!fft_plan_1d(Nx, px) || !fft_plan_1d(Ny, py)) throw MsError{NBPM_ERR_ARG, "FFT plan too deep"};

		MCK(cudaSetDevice(in.device));
		int optin = 0;
		MCK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, in.device));
		smem_limit = (size_t)optin;
		size_t per_line = 2 * (size_t)(std::max(Nx, Ny) + 1) * sizeof(cx<double>);
		if(per_line > smem_limit)
			throw MsError{NBPM_ERR_SIZE, "mesh dimension " + std::to_string(std::max(Nx, Ny)) +
				" exceeds the shared-memory FFT line limit"};
		MCK(cudaFuncSetAttribute(k_fft_lines<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_limit));
		MCK(cudaFuncSetAttribute(k_focus_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_limit));
		MCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
		for(auto& e : ev) MCK(cudaEventCreate(&e));
		const size_t nlq = (size_t)Nl * Nq * N;
		dwl.alloc(sizeof(double) * Nl);
		dnout.alloc(sizeof(double) * Nl);
		dqv.alloc(sizeof(double) * qv.size());
		tab.alloc(sizeof(double2) * nlq);
		filt.alloc(sizeof(cx<double>) * nlq);
		vals.alloc(sizeof(cx<double>) * nvals());
		foc.alloc(sizeof(cx<double>) * nvals());
		spec.alloc(sizeof(double) * N * Nl);
		dpre.alloc(sizeof(cx<double>) * 4 * Nl);
		dpost.alloc(sizeof(cx<double>) * 4 * Nl);
		bytes = (long long)(2 * sizeof(cx<double>) * nvals() + (sizeof(double2) + sizeof(cx<double>)) * nlq +
			sizeof(double) * N * Nl);
		MCK(cudaMemcpyAsync(dwl.p, wl.data(), sizeof(double) * Nl, cudaMemcpyHostToDevice, st));
		MCK(cudaMemcpyAsync(dnout.p, nout.data(), sizeof(double) * Nl, cudaMemcpyHostToDevice, st));
		MCK(cudaMemcpyAsync(dqv.p, qv.data(), sizeof(double) * qv.size(), cudaMemcpyHostToDevice, st));
		MCK(cudaMemsetAsync(vals.p, 0, sizeof(cx<double>) * nvals(), st));
		MCK(cudaMemsetAsync(foc.p, 0, sizeof(cx<double>) * nvals(), st));
		twiddles(twx, Nx);
		twiddles(twy, Ny);
		const int T = 256;
		k_objective_table<<<(unsigned)((nlq + T - 1) / T), T, 0, st>>>(Nx, Ny, Nl, Nq, dx, dy, dwl.as<double>(),
			dnout.as<double>(), dqv.as<double>(), tab.as<double2>());
		MCK(cudaGetLastError());
		MCK(cudaStreamSynchronize(st));
	}

	// x-line FFT of every plane, from src (null: in place) into foc.
	void fft_rows(const cx<double>* src, int sign) {
		FftPlan1D px;
		fft_plan_1d(Nx, px);
		size_t per_line = 2 * (size_t)(Nx + 1) * sizeof(cx<double>);
		int lpb = (int)std::max<size_t>(1, std::min<size_t>(64, (size_t)(48 * 1024) / per_line));
		lpb = std::max(1, std::min(lpb, (int)(smem_limit / per_line)));
		int nlines = Nl * Nq * 4 * Ny;
		int blocks = (nlines + lpb - 1) / lpb;
		int threads = std::min(256, std::max(32, ((lpb * Nx / 2) + 31) / 32 * 32));
		k_fft_lines<double><<<blocks, threads, per_line * lpb, st>>>(foc.as<cx<double>>(), src, px, nlines, Ny, N,
			Nx, 1, lpb, twx.as<cx<double>>(), sign);
	}

	void focus(double z_focus, double NA_obj) {
		MCK(cudaSetDevice(P.device));
		NA = std::max(0.0, std::min(P.max_NA_objective, NA_obj));
		z = z_focus;
		double zf = z + NA * NA * P.zfoc_NA_corr;
		double a = std::fabs(zf);
		const size_t nlq = (size_t)Nl * Nq * N;
		MCK(cudaEventRecord(ev[0], st));
		const int T = 256;
		k_focus_filter<<<(unsigned)((nlq + T - 1) / T), T, 0, st>>>(N, Nl, Nq, NA, a, zf < 0, 1.0 / (double)N,
			dwl.as<double>(), tab.as<double2>(), filt.as<cx<double>>());
		if(Nx > 1) fft_rows(vals.as<cx<double>>(), -1);
		else MCK(cudaMemcpyAsync(foc.p, vals.p, sizeof(cx<double>) * nvals(), cudaMemcpyDeviceToDevice, st));
		FftPlan1D py;
		fft_plan_1d(Ny, py);
		size_t per_line = 2 * (size_t)(Ny + 1) * sizeof(cx<double>);
		int lpb = (int)std::max<size_t>(1, std::min<size_t>(16, smem_limit / per_line));
		int nlines = Nl * Nq * 4 * Nx;
		int blocks = (nlines + lpb - 1) / lpb;
		int threads = std::min(256, std::max(32, ((lpb * Ny / 2) + 31) / 32 * 32));
		k_focus_cols<<<blocks, threads, per_line * lpb, st>>>(foc.as<cx<double>>(), py, nlines, Nx, N, lpb,
			twy.as<cx<double>>(), filt.as<cx<double>>());
		if(Nx > 1) fft_rows(nullptr, +1);
		MCK(cudaGetLastError());
		MCK(cudaEventRecord(ev[1], st));
		MCK(cudaEventSynchronize(ev[1]));
		MCK(cudaEventElapsedTime(&focus_ms, ev[0], ev[1]));
	}

	void spectrum(const nbpm_viewer_settings& vs, double* out_host, double* out_dev) {
		MCK(cudaSetDevice(P.device));
		for(int k : {vs.lower_waveplate, vs.upper_waveplate})
			if(k < NBPM_WAVEPLATE_NONE || k > NBPM_WAVEPLATE_TINT) throw MsError{NBPM_ERR_ARG, "unknown waveplate type"};
		Weights W = koehler_weights(vs.NA_condenser, P.max_NA_condenser, P.N_radial_wavevectors, P.koehler_1D);
		if(W.q_start < 0 || W.q_start + (int)W.w.size() > Nq)
			throw MsError{NBPM_ERR_SIZE, "condenser aperture needs wavevectors " + std::to_string(W.q_start) + ".." +
				std::to_string(W.q_start + (int)W.w.size() - 1) + " but only " + std::to_string(Nq) + " are set"};
		bool plain = !vs.polariser && !vs.analyser && vs.lower_waveplate == NBPM_WAVEPLATE_NONE &&
			vs.upper_waveplate == NBPM_WAVEPLATE_NONE;
		std::vector<cx<double>> pre(4 * (size_t)Nl), post(4 * (size_t)Nl);
		for(int l = 0; l < Nl; l++) {
			M2 a = eye(), b = eye();
			if(vs.polariser) a = polariser(vs.polariser_angle);
			if(vs.lower_waveplate != NBPM_WAVEPLATE_NONE) a = mul(waveplate(vs.lower_waveplate, vs.lower_waveplate_angle, wl[l]), a);
			if(vs.upper_waveplate != NBPM_WAVEPLATE_NONE) b = waveplate(vs.upper_waveplate, vs.upper_waveplate_angle, wl[l]);
			if(vs.analyser) b = mul(polariser(vs.analyser_angle), b);
			for(int i = 0; i < 4; i++) {
				pre[4 * l + i] = mk(a.a[i].real(), a.a[i].imag());
				post[4 * l + i] = mk(b.a[i].real(), b.a[i].imag());
			}
		}
		if(W.w.size() > nw_cap) {
			nw_cap = W.w.size();
			dw.alloc(sizeof(double) * nw_cap);
		}
		MCK(cudaMemcpyAsync(dw.p, W.w.data(), sizeof(double) * W.w.size(), cudaMemcpyHostToDevice, st));
		MCK(cudaMemcpyAsync(dpre.p, pre.data(), sizeof(cx<double>) * pre.size(), cudaMemcpyHostToDevice, st));
		MCK(cudaMemcpyAsync(dpost.p, post.data(), sizeof(cx<double>) * post.size(), cudaMemcpyHostToDevice, st));
		double* o = out_dev ? out_dev : spec.as<double>();
		MCK(cudaEventRecord(ev[2], st));
		const int T = 256;
		k_spectrum<<<dim3((unsigned)((N + T - 1) / T), (unsigned)Nl), T, 0, st>>>(foc.as<cx<double>>(), N, Nl, Nq,
			W.q_start, (int)W.w.size(), dw.as<double>(), dpre.as<cx<double>>(), dpost.as<cx<double>>(), plain ? 1 : 0, o);
		MCK(cudaGetLastError());
		MCK(cudaEventRecord(ev[3], st));
		if(out_host) MCK(cudaMemcpyAsync(out_host, o, sizeof(double) * N * Nl, cudaMemcpyDeviceToHost, st));
		MCK(cudaStreamSynchronize(st));
		MCK(cudaEventElapsedTime(&spectrum_ms, ev[2], ev[3]));
	}
};

}  // namespace nbpm

using namespace nbpm;

struct nbpm_microscope {
	std::unique_ptr<Microscope> m;
};

#define MS_GUARD(...)                                                                  \
	try { __VA_ARGS__ }                                                                \
	catch(MsError& e) { set_last_error(e.msg); return e.code; }                        \
	catch(std::bad_alloc&) { set_last_error("host out of memory"); return NBPM_ERR_MEMORY; } \
	catch(std::exception& e) { set_last_error(e.what()); return NBPM_ERR_INTERNAL; }   \
	catch(...) { set_last_error("unknown exception"); return NBPM_ERR_INTERNAL; }

extern "C" {

void nbpm_default_viewer_settings(nbpm_viewer_settings* s) {
	if(!s) return;
	std::memset(s, 0, sizeof(*s));
}

int nbpm_microscope_create(const nbpm_microscope_params* params, nbpm_microscope** out) {
	MS_GUARD({
		if(!params || !out) { set_last_error("null argument"); return NBPM_ERR_ARG; }
		*out = nullptr;
		std::unique_ptr<nbpm_microscope> h(new nbpm_microscope());
		h->m.reset(new Microscope());
		h->m->setup(*params);
		*out = h.release();
		return 0;
	})
}

int nbpm_microscope_destroy(nbpm_microscope* h) {
	delete h;
	return 0;
}

int nbpm_microscope_shape(const nbpm_microscope* h, int* n_wavelengths, int* n_wavevectors, int* Ny, int* Nx) {
	if(!h) { set_last_error("null microscope"); return NBPM_ERR_ARG; }
	if(n_wavelengths) *n_wavelengths = h->m->Nl;
	if(n_wavevectors) *n_wavevectors = h->m->Nq;
	if(Ny) *Ny = h->m->Ny;
	if(Nx) *Nx = h->m->Nx;
	return 0;
}

int nbpm_microscope_wavevectors(const nbpm_microscope* h, double* out, int n) {
	if(!h || !out) { set_last_error("null argument"); return NBPM_ERR_ARG; }
	if(n != h->m->Nq) { set_last_error("wavevector buffer must hold n_wavevectors x 2 values"); return NBPM_ERR_SIZE; }
	std::memcpy(out, h->m->qv.data(), sizeof(double) * h->m->qv.size());
	return 0;
}

int nbpm_microscope_set_fields(nbpm_microscope* h, const double* vals, long long n_vals) {
	MS_GUARD({
		if(!h || !vals) { set_last_error("null argument"); return NBPM_ERR_ARG; }
		Microscope& m = *h->m;
		if((size_t)n_vals != m.nvals()) { set_last_error("Wrong shape for the optical field ndarray"); return NBPM_ERR_SIZE; }
		MCK(cudaSetDevice(m.P.device));
		MCK(cudaMemcpyAsync(m.vals.p, vals, sizeof(cx<double>) * m.nvals(), cudaMemcpyHostToDevice, m.st));
		MCK(cudaStreamSynchronize(m.st));
		return 0;
	})
}

int nbpm_microscope_set_fields_from_plan(nbpm_microscope* h, nbpm_plan* plan, int sample) {
	MS_GUARD({
		if(!h || !plan) { set_last_error("null argument"); return NBPM_ERR_ARG; }
		Microscope& m = *h->m;
		PlanFieldsView v;
		if(!plan_fields_view(plan, sample, v)) { set_last_error("sample index out of range"); return NBPM_ERR_ARG; }
		if(v.Nx != m.Nx || v.Ny != m.Ny || v.Nl != m.Nl || v.Nq != m.Nq || v.n != m.nvals())
			{ set_last_error("plan sample and microscope have different field shapes"); return NBPM_ERR_SIZE; }
		if(v.device != m.P.device) { set_last_error("plan and microscope are on different devices"); return NBPM_ERR_ARG; }
		MCK(cudaSetDevice(m.P.device));
		MCK(cudaStreamSynchronize(v.stream));
		if(v.fp32) {
			k_widen_f32<<<(unsigned)((v.n + 255) / 256), 256, 0, m.st>>>(v.n, static_cast<const cx<float>*>(v.ptr),
				m.vals.as<cx<double>>());
			MCK(cudaGetLastError());
		}
		else MCK(cudaMemcpyAsync(m.vals.p, v.ptr, sizeof(cx<double>) * v.n, cudaMemcpyDeviceToDevice, m.st));
		MCK(cudaStreamSynchronize(m.st));
		return 0;
	})
}

int nbpm_microscope_focus(nbpm_microscope* h, double z_focus, double NA_objective) {
	MS_GUARD({
		if(!h) { set_last_error("null microscope"); return NBPM_ERR_ARG; }
		h->m->focus(z_focus, NA_objective);
		return 0;
	})
}

int nbpm_microscope_get_focused(nbpm_microscope* h, double* out, long long n_vals) {
	MS_GUARD({
		if(!h || !out) { set_last_error("null argument"); return NBPM_ERR_ARG; }
		Microscope& m = *h->m;
		if((size_t)n_vals != m.nvals()) { set_last_error("focused buffer has the wrong size"); return NBPM_ERR_SIZE; }
		MCK(cudaSetDevice(m.P.device));
		MCK(cudaMemcpyAsync(out, m.foc.p, sizeof(cx<double>) * m.nvals(), cudaMemcpyDeviceToHost, m.st));
		MCK(cudaStreamSynchronize(m.st));
		return 0;
	})
}

int nbpm_microscope_spectrum(nbpm_microscope* h, const nbpm_viewer_settings* vs, double* spectrum, long long n) {
	MS_GUARD({
		if(!h || !vs || !spectrum) { set_last_error("null argument"); return NBPM_ERR_ARG; }
		Microscope& m = *h->m;
		if(n != m.N * m.Nl) { set_last_error("spectrum buffer must hold Ny*Nx*n_wavelengths values"); return NBPM_ERR_SIZE; }
		m.spectrum(*vs, spectrum, nullptr);
		return 0;
	})
}

int nbpm_microscope_timing(const nbpm_microscope* h, double* focus_ms, double* spectrum_ms, long long* device_bytes) {
	if(!h) { set_last_error("null microscope"); return NBPM_ERR_ARG; }
	if(focus_ms) *focus_ms = h->m->focus_ms;
	if(spectrum_ms) *spectrum_ms = h->m->spectrum_ms;
	if(device_bytes) *device_bytes = h->m->bytes;
	return 0;
}

}  // extern "C"
