// Batched 2-D complex FFTs and the screen-plane Fourier filter.
//
// The reference transforms each wavelength's 4*Nq planes (Ny, Nx) with FFTW
// (OpticalFieldCollection.cpp:62-71: unnormalised, full Nx including the duplicated
// periodic column) and multiplies by the 2x2 transfer filter of ScreenOutput.cpp:226-302.
// Here a line FFT is a shared-memory Stockham autosort transform, mixed radix: stages of
// radix 4, 2, 3, 5, 7 and a generic prime radix. A block transforms `lpb` lines; rows
// (stride 1) load with the element index fastest, columns (stride Nx) load adjacent columns
// together so global accesses stay coalesced. Twiddles W_n^k = exp(-2*pi*i*k/n) come from a
// table computed on the host in FP64 with std::cos/std::sin.
#pragma once

#include "cplx.cuh"

namespace nbpm {

constexpr int FFT_MAX_STAGES = 24;

struct FftPlan1D {
	int n;
	int nst;
	int radix[FFT_MAX_STAGES];
};

// Radix sequence for a length-n line: 4s, then 2s, then odd primes in increasing order.
// Returns false when n needs more than FFT_MAX_STAGES stages.
inline bool fft_plan_1d(int n, FftPlan1D& P) {
	P.n = n;
	P.nst = 0;
	auto push = [&](int r) {
		if(P.nst >= FFT_MAX_STAGES) return false;
		P.radix[P.nst++] = r;
		return true;
	};
	while(n % 4 == 0 && n > 1) { if(!push(4)) return false; n /= 4; }
	while(n % 2 == 0) { if(!push(2)) return false; n /= 2; }
	for(int p = 3; n > 1 && p * p <= n; p += 2)
		while(n % p == 0) { if(!push(p)) return false; n /= p; }
	if(n > 1 && !push(n)) return false;
	return true;
}

template <typename R>
__device__ __forceinline__ cx<R> tw_get(const cx<R>* tw, int idx, int sign) {
	cx<R> w = tw[idx];
	return sign > 0 ? conj(w) : w;
}

// Mixed-radix Stockham stages on nl lines held in shared memory (pitch n+1): `in` holds the
// input; returns the buffer (in or out) that holds the transform. Ends with __syncthreads().
template <typename R>
__device__ cx<R>* fft_stages(cx<R>* in, cx<R>* out, const FftPlan1D& P, int nl, const cx<R>* __restrict__ tw,
		int sign) {
	const int n = P.n, pitch = n + 1;
	int Ns = 1;
	for(int st = 0; st < P.nst; st++) {
		int p = P.radix[st];
		int nb = n / p;  // butterflies per line
		int span = n / (Ns * p);  // twiddle index scale
		for(int e = threadIdx.x; e < nl * nb; e += blockDim.x) {
			int li = e / nb, j = e % nb;
			const cx<R>* I = in + li * pitch;
			cx<R>* O = out + li * pitch;
			int k = j % Ns;
			int obase = (j / Ns) * Ns * p + k;
			cx<R> v[8];
			if(p <= 8) {
				for(int r = 0; r < p; r++) {
					cx<R> x = I[j + r * nb];
					if(r && k) x = x * tw_get(tw, r * k * span, sign);
					v[r] = x;
				}
				if(p == 2) {
					O[obase] = v[0] + v[1];
					O[obase + Ns] = v[0] - v[1];
				}
				else if(p == 4) {
					cx<R> a = v[0] + v[2], b = v[0] - v[2];
					cx<R> c = v[1] + v[3], d = v[1] - v[3];
					// multiply d by -i (forward) or +i (backward)
					cx<R> dj = sign > 0 ? mk<R>(-d.y, d.x) : mk<R>(d.y, -d.x);
					O[obase] = a + c;
					O[obase + Ns] = b + dj;
					O[obase + 2 * Ns] = a - c;
					O[obase + 3 * Ns] = b - dj;
				}
				else {
					int wstep = n / p;
					for(int s = 0; s < p; s++) {
						cx<R> acc = v[0];
						for(int r = 1; r < p; r++)
							acc += v[r] * tw_get(tw, ((r * s) % p) * wstep, sign);
						O[obase + s * Ns] = acc;
					}
				}
			}
			else {
				// generic prime radix: direct p-point DFT (inputs re-read from shared memory)
				int wstep = n / p;
				for(int s = 0; s < p; s++) {
					cx<R> acc = mk<R>(0, 0);
					for(int r = 0; r < p; r++) {
						cx<R> x = I[j + r * nb];
						if(r && k) x = x * tw_get(tw, (int)(((long long)r * k * span) % n), sign);
						acc += x * tw_get(tw, (int)(((long long)r * s % p) * wstep), sign);
					}
					O[obase + s * Ns] = acc;
				}
			}
		}
		__syncthreads();
		cx<R>* t = in; in = out; out = t;
		Ns *= p;
	}
	return in;
}

// Transform `nlines` lines of length P.n. Line l starts at base(l) = (l / lines_per_plane)
// * plane_stride + (l % lines_per_plane) * line_stride and its elements are elem_stride apart.
// Reads from `src` (data when null) and writes to `data`.
template <typename R>
static __global__ void k_fft_lines(cx<R>* data, const cx<R>* src, FftPlan1D P, int nlines, int lines_per_plane,
		long long plane_stride, long long line_stride, long long elem_stride, int lpb,
		const cx<R>* __restrict__ tw, int sign) {
	extern __shared__ unsigned char smem_raw[];
	cx<R>* sA = reinterpret_cast<cx<R>*>(smem_raw);
	const int n = P.n, pitch = n + 1;
	cx<R>* sB = sA + (size_t)lpb * pitch;
	int l0 = blockIdx.x * lpb;
	int nl = min(lpb, nlines - l0);
	if(nl <= 0) return;
	const cx<R>* in_data = src ? src : data;
	auto base = [&](int l) {
		return (long long)(l / lines_per_plane) * plane_stride + (long long)(l % lines_per_plane) * line_stride;
	};
	int tot = nl * n;
	if(elem_stride == 1) {
		for(int e = threadIdx.x; e < tot; e += blockDim.x) {
			int li = e / n, i = e % n;
			sA[li * pitch + i] = in_data[base(l0 + li) + i];
		}
	}
	else {
		for(int e = threadIdx.x; e < tot; e += blockDim.x) {
			int li = e % nl, i = e / nl;
			sA[li * pitch + i] = in_data[base(l0 + li) + (long long)i * elem_stride];
		}
	}
	__syncthreads();
	cx<R>* in = fft_stages<R>(sA, sB, P, nl, tw, sign);
	if(elem_stride == 1) {
		for(int e = threadIdx.x; e < tot; e += blockDim.x) {
			int li = e / n, i = e % n;
			data[base(l0 + li) + i] = in[li * pitch + i];
		}
	}
	else {
		for(int e = threadIdx.x; e < tot; e += blockDim.x) {
			int li = e % nl, i = e / nl;
			data[base(l0 + li) + (long long)i * elem_stride] = in[li * pitch + i];
		}
	}
}

// Screen filter of ScreenOutput::assemble_fourier_filter (ScreenOutput.cpp:226-302), FP64,
// applied to both polarisation slots of every (group, q) with the 1/(Nx*Ny) scaling of
// apply_no_export (:212-219). q0_sqr is |q0| as in :252.
struct ScreenParams {
	int Nx, Ny, Nq, n_iso;
	double dx, dy, NA, z_foc;
	double thick[8];
	double index[9];  // iso layer indices; last entry replaced per group by nout(lambda)
};

template <typename R>
__global__ void k_screen_filter(cx<R>* F, ScreenParams sp, int g0, const double* __restrict__ wl,
		const double* __restrict__ nout, const double* __restrict__ qv) {
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	int Nx = sp.Nx, Ny = sp.Ny, N = Nx * Ny;
	if(p >= N) return;
	int gq = blockIdx.y;            // group-local (g, q)
	int g = gq / sp.Nq, q = gq % sp.Nq;
	int ix = p % Nx, iy = p / Nx;
	const double PI_REF = 3.1415926535897932;
	double lam = wl[g0 + g];
	double k0 = 2 * PI_REF / lam;
	double kx = (ix < double(Nx / 2.)) ? 2 * PI_REF * ix / (sp.dx * Nx) : -2 * PI_REF * (Nx - ix) / (sp.dx * Nx);
	double ky = (iy < double(Ny / 2.)) ? 2 * PI_REF * iy / (sp.dy * Ny) : -2 * PI_REF * (Ny - iy) / (sp.dy * Ny);
	double qx0 = qv[2 * q], qy0 = qv[2 * q + 1];
	double q0 = kx / k0 + qx0, q1 = ky / k0 + qy0;
	double qn = sqrt(q0 * q0 + q1 * q1);
	double qn2 = qn * qn;
	double q0s = sqrt(qx0 * qx0 + qy0 * qy0);
	cx<double> M[2][2] = {{mk(0.0, 0.0), mk(0.0, 0.0)}, {mk(0.0, 0.0), mk(0.0, 0.0)}};
	if(qn < sp.NA) {
		double n_out = nout[g0 + g];
		cx<double> T[4][4];
		for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) T[a][b] = mk(a == b ? 1.0 : 0.0, 0.0);
		for(int l = 0; l < sp.n_iso; l++) {
			double np = sp.index[l];
			double nn = (l + 1 < sp.n_iso) ? sp.index[l + 1] : n_out;
			double neff = sqrt(np * np - qn2), nneff = sqrt(nn * nn - qn2);
			double im[2][2] = {{neff + q0 * q0 / neff, q0 * q1 / neff}, {q0 * q1 / neff, neff + q1 * q1 / neff}};
			double ni[2][2] = {{(1 - (q0 / nn) * (q0 / nn)) / nneff, -q0 * q1 / (nn * nn * nneff)},
				{-q0 * q1 / (nn * nn * nneff), (1 - (q1 / nn) * (q1 / nn)) / nneff}};
			double tp[2][2], tm[2][2];
			for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++)
				tp[a][b] = 0.5 * ((a == b ? 1. : 0.) + ni[a][0] * im[0][b] + ni[a][1] * im[1][b]);
			for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) tm[a][b] = (a == b ? 1. : 0.) - tp[a][b];
			double ph = (neff - sqrt(np * np - q0s)) * k0 * sp.thick[l];
			cx<double> gg = mk(cos(ph), sin(ph)), gc = conj(gg);
			cx<double> Lm[4][4];
			for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) {
				Lm[a][b] = tp[a][b] * gg;
				Lm[a][b + 2] = tm[a][b] * gc;
				Lm[a + 2][b] = tm[a][b] * gg;
				Lm[a + 2][b + 2] = tp[a][b] * gc;
			}
			cx<double> T2[4][4];
			for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) {
				cx<double> s = mk(0.0, 0.0);
				for(int c = 0; c < 4; c++) s += Lm[a][c] * T[c][b];
				T2[a][b] = s;
			}
			for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) T[a][b] = T2[a][b];
		}
		cx<double> det = T[2][2] * T[3][3] - T[2][3] * T[3][2];
		cx<double> tmp[2][2] = {{cdiv(T[3][3], det), cdiv(-T[2][3], det)}, {cdiv(-T[3][2], det), cdiv(T[2][2], det)}};
		double ph = (sqrt(n_out * n_out - qn2) - sqrt(n_out * n_out - q0s)) * k0 * sp.z_foc;
		cx<double> e = mk(cos(ph), sin(ph));
		for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) {
			cx<double> s = mk(0.0, 0.0);
			for(int c = 0; c < 2; c++) for(int d = 0; d < 2; d++) s += T[a][c + 2] * tmp[c][d] * T[d + 2][b];
			M[a][b] = (T[a][b] - s) * e;
		}
	}
	double inv = 1.0 / double(N);
	for(int pol = 0; pol < 2; pol++) {
		size_t slot = (size_t)pol + 2 * ((size_t)q + (size_t)sp.Nq * g);
		cx<R>* f = F + slot * 2 * N + p;
		cx<double> a = cvt<double>(f[0]), b = cvt<double>(f[N]);
		cx<double> t0 = M[0][0] * a + M[0][1] * b;
		cx<double> t1 = M[1][0] * a + M[1][1] * b;
		f[0] = cvt<R>(t0 * inv);
		f[N] = cvt<R>(t1 * inv);
	}
}

}  // namespace nbpm
