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
	// transfer matrices in the plan's precision (FP32 mode: FP32, within its error budget)
	using T = R;
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	int Nx = sp.Nx, Ny = sp.Ny, N = Nx * Ny;
	if(p >= N) return;
	int gq = blockIdx.y;            // group-local (g, q)
	int g = gq / sp.Nq, q = gq % sp.Nq;
	int ix = p % Nx, iy = p / Nx;
	const double PI_REF = 3.1415926535897932;
	const T k0 = (T)(2 * PI_REF / wl[g0 + g]);
	const double kx = (ix < double(Nx / 2.)) ? 2 * PI_REF * ix / (sp.dx * Nx) : -2 * PI_REF * (Nx - ix) / (sp.dx * Nx);
	const double ky = (iy < double(Ny / 2.)) ? 2 * PI_REF * iy / (sp.dy * Ny) : -2 * PI_REF * (Ny - iy) / (sp.dy * Ny);
	// the aperture test in FP64 in both modes, so that no mode near |q| = NA flips in or out
	const double k0d = 2 * PI_REF / wl[g0 + g];
	const double q0d = (double)kx / k0d + qv[2 * q], q1d = (double)ky / k0d + qv[2 * q + 1];
	const double qnd = sqrt(q0d * q0d + q1d * q1d);
	const T qx0 = (T)qv[2 * q], qy0 = (T)qv[2 * q + 1];
	const T q0 = (T)q0d, q1 = (T)q1d;
	const T qn = (T)qnd;
	const T qn2 = qn * qn;
	const T q0s = sqrt(qx0 * qx0 + qy0 * qy0);
	const cx<T> zero = mk<T>(0, 0);
	cx<T> M[2][2] = {{zero, zero}, {zero, zero}};
	if(qnd < sp.NA) {
		const T n_out = (T)nout[g0 + g];
		cx<T> TM[4][4];
		for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) TM[a][b] = mk<T>(a == b ? 1 : 0, 0);
		for(int l = 0; l < sp.n_iso; l++) {
			const T np = (T)sp.index[l];
			const T nn = (l + 1 < sp.n_iso) ? (T)sp.index[l + 1] : n_out;
			const T neff = sqrt(np * np - qn2), nneff = sqrt(nn * nn - qn2);
			const T im[2][2] = {{neff + q0 * q0 / neff, q0 * q1 / neff}, {q0 * q1 / neff, neff + q1 * q1 / neff}};
			const T ni[2][2] = {{(1 - (q0 / nn) * (q0 / nn)) / nneff, -q0 * q1 / (nn * nn * nneff)},
				{-q0 * q1 / (nn * nn * nneff), (1 - (q1 / nn) * (q1 / nn)) / nneff}};
			T tp[2][2], tm[2][2];
			for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++)
				tp[a][b] = (T)0.5 * ((a == b ? (T)1 : (T)0) + ni[a][0] * im[0][b] + ni[a][1] * im[1][b]);
			for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) tm[a][b] = (a == b ? (T)1 : (T)0) - tp[a][b];
			const T ph = (neff - sqrt(np * np - q0s)) * k0 * (T)sp.thick[l];
			const cx<T> gg = mk<T>(cos(ph), sin(ph)), gc = conj(gg);
			cx<T> Lm[4][4];
			for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) {
				Lm[a][b] = tp[a][b] * gg;
				Lm[a][b + 2] = tm[a][b] * gc;
				Lm[a + 2][b] = tm[a][b] * gg;
				Lm[a + 2][b + 2] = tp[a][b] * gc;
			}
			cx<T> T2[4][4];
			for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) {
				cx<T> s = zero;
				for(int c = 0; c < 4; c++) s += Lm[a][c] * TM[c][b];
				T2[a][b] = s;
			}
			for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) TM[a][b] = T2[a][b];
		}
		const cx<T> det = TM[2][2] * TM[3][3] - TM[2][3] * TM[3][2];
		const cx<T> tmp[2][2] = {{cdiv(TM[3][3], det), cdiv(-TM[2][3], det)}, {cdiv(-TM[3][2], det), cdiv(TM[2][2], det)}};
		const T ph = (sqrt(n_out * n_out - qn2) - sqrt(n_out * n_out - q0s)) * k0 * (T)sp.z_foc;
		const cx<T> e = mk<T>(cos(ph), sin(ph));
		for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) {
			cx<T> s = zero;
			for(int c = 0; c < 2; c++) for(int d = 0; d < 2; d++) s += TM[a][c + 2] * tmp[c][d] * TM[d + 2][b];
			M[a][b] = (TM[a][b] - s) * e;
		}
	}
	const T inv = (T)(1.0 / double(N));
	for(int pol = 0; pol < 2; pol++) {
		size_t slot = (size_t)pol + 2 * ((size_t)q + (size_t)sp.Nq * g);
		cx<R>* f = F + slot * 2 * N + p;
		const cx<T> a = f[0], b = f[N];
		const cx<T> t0 = M[0][0] * a + M[0][1] * b;
		const cx<T> t1 = M[1][0] * a + M[1][1] * b;
		f[0] = t0 * inv;
		f[N] = t1 * inv;
	}
}

}  // namespace nbpm
