// sm_103a kernels of the bpm z-stepping loop.
//
// Data layout in HBM (one sample):
//   director  dir[iz][iy][ix][c]            FP64, c < 3 (director) or 6 (Q-tensor)
//   fields    F[slot][comp][iy][ix]          cx<R>; slot = pol + 2*(q + Nq*lambda): the same
//                                            order as the (Nl,Nq,4,Ny,Nx) user buffer
//   eps ring  Q[2][group][NQ][iy][ix]        FP64 per-voxel derived permittivity, planes iz
//                                            and iz+1 of every wavelength group
//   coef      C[group][p/32][NCOEF][p%32]    cx<R>: 3 phase-operator entries and the 40
//                                            entries of mu*R (DX, DY, DXDY stencils x 4 blocks),
//                                            p = iy*Nx + ix, in tiles of 32 points (cidx)
//   factors   X/Y[group][comp][NFAC][p]      cx<R>: pre-factored periodic line solves
// A "group" is one wavelength: every (q, pol) slot of the group shares eps, R, the phase
// operator and the line-solve factorisations.
#pragma once

#include <cstdint>

#include "cplx.cuh"

namespace nbpm {

// Per-voxel derived permittivity components (PermittivityTensorField.cpp:3-99).
enum { Q_XXTR = 0, Q_YYTR, Q_XYTR, Q_XXS, Q_YYS, Q_XYS, Q_VX, Q_VY, Q_IZZ, NQ };
// Coefficient planes: phase operator (xx, yy, xy), then mu*R stencils.
enum { C_PH = 0, C_DX = 3, C_DY = 15, C_DXDY = 27, NCOEF = 43 };
// A group's coefficient set is stored in tiles of 32 points with every plane of a tile together:
// entry (plane k, point p) at ((p / 32) * NCOEF + k) * 32 + p % 32, NCOEF * ceil(N / 32) * 32
// entries per group. The planes a kernel reads at one point are then fixed multiples of 32
// entries apart (compile-time offsets from one address), and 32 consecutive points of a plane
// starting at a multiple of 32 are one contiguous segment.
__host__ __device__ __forceinline__ size_t coef_set_size(int N) { return (size_t)NCOEF * (((size_t)N + 31) & ~(size_t)31); }
__host__ __device__ __forceinline__ size_t cidx(int k, int p) { return ((size_t)(p >> 5) * NCOEF + k) * 32 + (p & 31); }
// FP64 copies of the diagonal-block stencils used by the line factorisations:
// index dir*6 + comp*3 + k (dir 0 = DX, 1 = DY; comp 0 = block 00, 1 = block 11).
enum { NDIAG = 12 };
// Line-solve factor planes.
// F_A = alpha_i = -inf_i/beta_i (forward recurrence d_i = alpha_i d_{i-1} + b_i/beta_i),
// F_RB = 1/beta_i, F_W = w_i, F_C = -gamma_i (backward recurrence), F_COR = corr_i.
enum { F_A = 0, F_RB, F_W, F_C, F_COR, NFAC };

struct GroupParams {
	double wavelength, k0, dX, dY, dZ;
	double no, ne, ne_imag, nhost, nin, nout_fresnel;
	double absorp_im;  // imaginary part of 1 + i*ne_imag/(ne-no)
	double nref;
};

struct ShiftParams {
	int active;       // 0: identity (q = 0)
	int msx, msy;     // integer parts of the shifts
	double wx[4], wy[4];
	double ph_re, ph_im;
	// the same weights and phase factor rounded to FP32 (the FP32 transition reads these instead of
	// converting the FP64 values at each use)
	float fwx[4], fwy[4];
	float fph_re, fph_im;
};

// Shift weights and phase factor in the arithmetic type R.
template <typename R>
struct ShiftW {
	R wx[4], wy[4];
	cx<R> ph;
	__device__ __forceinline__ explicit ShiftW(const ShiftParams& P) {
#pragma unroll
		for(int k = 0; k < 4; k++) {
			wx[k] = sizeof(R) == sizeof(float) ? (R)P.fwx[k] : (R)P.wx[k];
			wy[k] = sizeof(R) == sizeof(float) ? (R)P.fwy[k] : (R)P.wy[k];
		}
		ph = sizeof(R) == sizeof(float) ? mk<R>((R)P.fph_re, (R)P.fph_im) : mk<R>((R)P.ph_re, (R)P.ph_im);
	}
};

struct Geom {
	int Nx, Ny, N;
	int Nz;
	int spg;          // slots per group = 2*Nq
	int Nq;
};

// ---------------------------------------------------------------------------------------
// Permittivity per voxel from the director or Q-tensor (PermittivityTensorField.cpp:19-99).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void eps_voxel(const double* __restrict__ dir, int fd, bool m,
		const GroupParams& gp, double e[6]) {
	double eps_perp = gp.no * gp.no;
	double eps_a = gp.ne * gp.ne - eps_perp;
	double eps_host = gp.nhost * gp.nhost;
	if(!m) {
		e[0] = e[1] = e[2] = eps_host;
		e[3] = e[4] = e[5] = 0;
		return;
	}
	if(fd == 3) {
		double n0 = dir[0], n1 = dir[1], n2 = dir[2];
		e[0] = eps_perp + eps_a * (n0 * n0);
		e[1] = eps_perp + eps_a * (n1 * n1);
		e[2] = eps_perp + eps_a * (n2 * n2);
		e[3] = eps_a * n0 * n1;
		e[4] = eps_a * n0 * n2;
		e[5] = eps_a * n1 * n2;
	}
	else {
		double ea = 2 * eps_a / 3, ei = eps_perp + eps_a / 3.;
		e[0] = ei + ea * dir[0];
		e[1] = ei + ea * dir[1];
		e[2] = ei + ea * dir[2];
		e[3] = ea * dir[3];
		e[4] = ea * dir[4];
		e[5] = ea * dir[5];
	}
}

__device__ __forceinline__ double neff_of(double xxtr, double yytr, double xytr) {
	double det = xxtr * yytr - xytr * xytr;
	double tr = 0.5 * (xxtr + yytr);
	if(tr * tr - det < 1e-8) return sqrt(tr);
	double r = sqrt(tr * tr - det);
	return (sqrt(tr + r) + sqrt(tr - r)) / 2.;
}

// neff of one voxel in FP32 arithmetic (the same formulas as eps_voxel + neff_of), for the nref
// mean of the FP32 mode.
__device__ __forceinline__ float neff_voxel_f(const double* __restrict__ dir, int fd, bool m, float eps_perp,
		float eps_a, float eps_host) {
	float e0, e1, e2, e3, e4, e5;
	if(!m) return sqrtf(eps_host);
	if(fd == 3) {
		float n0 = (float)dir[0], n1 = (float)dir[1], n2 = (float)dir[2];
		e0 = eps_perp + eps_a * (n0 * n0);
		e1 = eps_perp + eps_a * (n1 * n1);
		e2 = eps_perp + eps_a * (n2 * n2);
		e3 = eps_a * n0 * n1;
		e4 = eps_a * n0 * n2;
		e5 = eps_a * n1 * n2;
	}
	else {
		float ea = 2 * eps_a / 3, ei = eps_perp + eps_a / 3.f;
		e0 = ei + ea * (float)dir[0];
		e1 = ei + ea * (float)dir[1];
		e2 = ei + ea * (float)dir[2];
		e3 = ea * (float)dir[3];
		e4 = ea * (float)dir[4];
		e5 = ea * (float)dir[5];
	}
	float xx = e0 - (e4 * e4) / e2, yy = e1 - (e5 * e5) / e2, xy = e3 - e4 * e5 / e2;
	float det = xx * yy - xy * xy, tr = 0.5f * (xx + yy);
	if(tr * tr - det < 1e-8f) return sqrtf(tr);
	float r = sqrtf(tr * tr - det);
	return (sqrtf(tr + r) + sqrtf(tr - r)) / 2.f;
}

// One transverse plane of derived quantities for every group of the pass, computed and
// stored in the plan's precision Q (FP64 mode: FP64; FP32 mode: FP32).
template <typename Q>
static __global__ void k_eps_plane(const double* __restrict__ dir, int fd, const uint8_t* __restrict__ mask,
		int N, int iz, const GroupParams* __restrict__ gps, Q* __restrict__ out) {
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	int g = blockIdx.y;
	if(p >= N) return;
	size_t v = (size_t)iz * N + p;
	GroupParams gp = gps[g];
	const bool m = mask ? mask[v] != 0 : true;
	Q* o = out + (size_t)g * NQ * N + p;
	if(sizeof(Q) == sizeof(float)) {
		// FP32 mode: the same formulas in FP32 arithmetic
		const float ep = (float)(gp.no * gp.no), ea = (float)(gp.ne * gp.ne - gp.no * gp.no);
		const float eh = (float)(gp.nhost * gp.nhost);
		const double* d = dir + v * fd;
		float e0, e1, e2, e3, e4, e5;
		if(!m) { e0 = e1 = e2 = eh; e3 = e4 = e5 = 0.f; }
		else if(fd == 3) {
			float n0 = (float)d[0], n1 = (float)d[1], n2 = (float)d[2];
			e0 = ep + ea * (n0 * n0); e1 = ep + ea * (n1 * n1); e2 = ep + ea * (n2 * n2);
			e3 = ea * n0 * n1; e4 = ea * n0 * n2; e5 = ea * n1 * n2;
		}
		else {
			float a = 2 * ea / 3, ei = ep + ea / 3.f;
			e0 = ei + a * (float)d[0]; e1 = ei + a * (float)d[1]; e2 = ei + a * (float)d[2];
			e3 = a * (float)d[3]; e4 = a * (float)d[4]; e5 = a * (float)d[5];
		}
		float xx = e0 - (e4 * e4) / e2, yy = e1 - (e5 * e5) / e2, xy = e3 - e4 * e5 / e2;
		float det = xx * yy - xy * xy, tr = 0.5f * (xx + yy), ne;
		if(tr * tr - det < 1e-8f) ne = sqrtf(tr);
		else { float r = sqrtf(tr * tr - det); ne = (sqrtf(tr + r) + sqrtf(tr - r)) / 2.f; }
		o[Q_XXTR * N] = (Q)xx;
		o[Q_YYTR * N] = (Q)yy;
		o[Q_XYTR * N] = (Q)xy;
		o[Q_XXS * N] = (Q)(ne + (xx - yy) / (4 * ne));
		o[Q_YYS * N] = (Q)(ne + (yy - xx) / (4 * ne));
		o[Q_XYS * N] = (Q)(xy / (2 * ne));
		o[Q_VX * N] = (Q)(e4 / e2);
		o[Q_VY * N] = (Q)(e5 / e2);
		o[Q_IZZ * N] = (Q)(1.f / e2);
		return;
	}
	double e[6];
	eps_voxel(dir + v * fd, fd, m, gp, e);
	double xxtr = e[0] - (e[4] * e[4]) / e[2];
	double yytr = e[1] - (e[5] * e[5]) / e[2];
	double xytr = e[3] - e[4] * e[5] / e[2];
	double neff = neff_of(xxtr, yytr, xytr);
	o[Q_XXTR * N] = (Q)xxtr;
	o[Q_YYTR * N] = (Q)yytr;
	o[Q_XYTR * N] = (Q)xytr;
	o[Q_XXS * N] = (Q)(neff + (xxtr - yytr) / (4 * neff));
	o[Q_YYS * N] = (Q)(neff + (yytr - xxtr) / (4 * neff));
	o[Q_XYS * N] = (Q)(xytr / (2 * neff));
	o[Q_VX * N] = (Q)(e[4] / e[2]);
	o[Q_VY * N] = (Q)(e[5] / e[2]);
	o[Q_IZZ * N] = (Q)(1. / e[2]);
}

// Partial sums of neff over the volume for nref (PermittivityTensorField.cpp:183-211),
// in a fixed block order so the reduction is deterministic.
// FP32 mode (F32 = true): neff in FP32 arithmetic, summed in FP64.
template <bool F32>
static __global__ void k_neff_partial(const double* __restrict__ dir, int fd, const uint8_t* __restrict__ mask,
		size_t nvox, const GroupParams* __restrict__ gps, double* __restrict__ partial) {
	__shared__ double sh[256];
	int g = blockIdx.y;
	GroupParams gp = gps[g];
	double acc = 0;
	const float ep = (float)(gp.no * gp.no), ea = (float)(gp.ne * gp.ne - gp.no * gp.no), eh = (float)(gp.nhost * gp.nhost);
	for(size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (size_t)gridDim.x * blockDim.x) {
		if(F32) {
			acc += (double)neff_voxel_f(dir + v * fd, fd, mask ? mask[v] != 0 : true, ep, ea, eh);
			continue;
		}
		double e[6];
		eps_voxel(dir + v * fd, fd, mask ? mask[v] != 0 : true, gp, e);
		double xxtr = e[0] - (e[4] * e[4]) / e[2];
		double yytr = e[1] - (e[5] * e[5]) / e[2];
		double xytr = e[3] - e[4] * e[5] / e[2];
		acc += neff_of(xxtr, yytr, xytr);
	}
	sh[threadIdx.x] = acc;
	__syncthreads();
	for(int s = blockDim.x / 2; s > 0; s >>= 1) {
		if(threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
		__syncthreads();
	}
	if(threadIdx.x == 0) partial[(size_t)g * gridDim.x + blockIdx.x] = sh[0];
}

// ---------------------------------------------------------------------------------------
// Per-slab operator coefficients (FP64 in FP64 mode; in FP32 mode the phase operator stays
// FP64 and the stencil entries of mu*R are formed in FP32):
//  * phase operator exp(i*a*d) (PhaseEvolutionOperator.cpp:34-63)
//  * mu*R with R = i*W + (D*S^-1 + S^-1*D)/4, D = D0 + D1*K (ParaxialPrimaryEvolution-
//    Operator.cpp:212-490), written per stencil entry: S^-1 and K at the column point for
//    D*S^-1 and D1*K, S^-1 at the row point for S^-1*D, the walk-off split between row
//    and column points. D1 uses the reference's neighbour indices (ix==Nx-1 -> 1,
//    ix==0 -> Nx-2) while the stencil columns wrap with period Nx-1.
// ---------------------------------------------------------------------------------------
template <typename T>
struct CoefCtx {
	const T* A;
	const T* B;
	int N, Nx;
	T hmu, rxx, ryy, rxy, va0, va1;
	__device__ __forceinline__ T avg(int q, int x, int y) const {
		int i = x + Nx * y;
		return (A[q * N + i] + B[q * N + i]) / (T)2;
	}
	__device__ __forceinline__ T vsum(int a, int x, int y) const {
		int i = x + Nx * y, q = a == 0 ? Q_VX : Q_VY;
		return A[q * N + i] + B[q * N + i];
	}
	__device__ __forceinline__ void sinv(int x, int y, T& ixx, T& iyy, T& ixy) const {
		T exx = avg(Q_XXS, x, y), eyy = avg(Q_YYS, x, y), exy = avg(Q_XYS, x, y);
		T det = exx * eyy - exy * exy;
		ixx = eyy / det; iyy = exx / det; ixy = -exy / det;
	}
	// One stencil entry of mu*R for the 4 blocks (00, 01, 10, 11). D is the real 2x2 entry
	// of D at this (row, column) pair; dd is the first-derivative weight of the walk-off
	// (0 for none) acting on component bT.
	__device__ void entry(T D00, T D01, T D10, T D11, int cxp, int cyp,
			T dd, int bT, cx<T> out[4]) const {
		T re[4] = {0, 0, 0, 0}, im[4] = {0, 0, 0, 0};
		if(dd != 0) {
			T vb0 = vsum(0, cxp, cyp), vb1 = vsum(1, cxp, cyp);
			im[0 + bT] += dd * ((T)0.25 * va0);
			im[2 + bT] += dd * ((T)0.25 * va1);
			im[2 * bT + 0] += dd * ((T)0.25 * vb0);
			im[2 * bT + 1] += dd * ((T)0.25 * vb1);
		}
		T cxx, cyy, cxy;
		sinv(cxp, cyp, cxx, cyy, cxy);
		T Dm[2][2] = {{D00, D01}, {D10, D11}};
		const T q4 = (T)0.25;
		for(int a = 0; a < 2; a++) {
			re[2 * a] += q4 * Dm[a][0] * cxx;
			re[2 * a] += q4 * Dm[a][1] * cxy;
			re[2 * a + 1] += q4 * Dm[a][0] * cxy;
			re[2 * a + 1] += q4 * Dm[a][1] * cyy;
		}
		for(int b = 0; b < 2; b++) {
			re[b] += q4 * rxx * Dm[0][b];
			re[b] += q4 * rxy * Dm[1][b];
			re[2 + b] += q4 * rxy * Dm[0][b];
			re[2 + b] += q4 * ryy * Dm[1][b];
		}
		for(int b = 0; b < 4; b++) out[b] = mk(-hmu * im[b], hmu * re[b]);  // i*hmu*(re+i*im)
	}
};

// Phase operator of one point (PhaseEvolutionOperator.cpp:14-32) from eps planes A, B of the
// slab's two ends, in the arithmetic type T.
template <typename T>
__device__ __forceinline__ void phase_op(const T* A, const T* B, int N, int p, T w0, T w1, const GroupParams& gp,
		cx<T>& oxx, cx<T>& oyy, cx<T>& oxy) {
	T hz = (T)(0.5 * gp.dZ);
	T dxx = hz * (w0 * A[Q_XXS * N + p] + w1 * B[Q_XXS * N + p] - (T)gp.no);
	T dyy = hz * (w0 * A[Q_YYS * N + p] + w1 * B[Q_YYS * N + p] - (T)gp.no);
	T dxy = hz * (w0 * A[Q_XYS * N + p] + w1 * B[Q_XYS * N + p]);
	T diff = (dxx - dyy) / (T)2, tr = (dxx + dyy) / (T)2;
	T det = sqrt(dxy * dxy + diff * diff);
	cx<T> a = mk<T>((T)1, (T)gp.absorp_im);
	cx<T> sinc = mk<T>((T)1, (T)0);
	cx<T> e, c;
	if(sizeof(T) == sizeof(double)) {
		cx<double> ad = cvt<double>(a);
		if(!(fabs((double)det) < 1e-8)) {
			cx<double> sn = csin_d((double)det * ad);
			sinc = cvt<T>(mk(sn.x / (double)det, sn.y / (double)det));
		}
		e = cvt<T>(cexp_d(mk(-ad.y * (double)tr, ad.x * (double)tr)));  // exp(i*a*tr)
		c = cvt<T>(ccos_d((double)det * ad));
	}
	else {
		cx<float> af = cvt<float>(a);
		if(!(fabsf((float)det) < 1e-8f)) {
			cx<float> sn = csin_f((float)det * af);
			sinc = cvt<T>(mk(sn.x / (float)det, sn.y / (float)det));
		}
		e = cvt<T>(cexp_f(mk(-af.y * (float)tr, af.x * (float)tr)));
		c = cvt<T>(ccos_f((float)det * af));
	}
	cx<T> ids = mk<T>((T)0, diff) * sinc;
	oxx = e * (c + ids);
	oyy = e * (c - ids);
	oxy = ((e * mk<T>((T)0, (T)1)) * dxy) * sinc;
}

template <typename S>
__global__ void k_coef(const S* __restrict__ QA, const S* __restrict__ QB,
		const double* __restrict__ wts, int iz, Geom G, const GroupParams* __restrict__ gps,
		cx<S>* __restrict__ coef, cx<S>* __restrict__ diag) {
	typedef S T;  // arithmetic type of the eps planes, the phase operator and the R coefficients
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	int g = blockIdx.y;
	int N = G.N, Nx = G.Nx, Ny = G.Ny;
	if(p >= N) return;
	int ix = p % Nx, iy = p / Nx;
	const GroupParams gp = gps[g];
	const T* A = QA + (size_t)g * NQ * N;
	const T* B = QB + (size_t)g * NQ * N;
	cx<S>* C = coef + (size_t)g * coef_set_size(N);
	cx<S>* Dg = diag + (size_t)g * NDIAG * N + p;

	// Phase operator.
	{
		T w0 = (T)0.5, w1 = (T)0.5;
		if(wts) { size_t vi = (size_t)iz * N + p; w0 = (T)wts[2 * vi]; w1 = (T)wts[2 * vi + 1]; }
		cx<T> oxx, oyy, oxy;
		phase_op<T>(A, B, N, p, w0, w1, gp, oxx, oyy, oxy);
		C[cidx(C_PH + 0, p)] = oxx;
		C[cidx(C_PH + 1, p)] = oyy;
		C[cidx(C_PH + 2, p)] = oxy;
	}

	CoefCtx<T> X;
	X.A = A; X.B = B; X.N = N; X.Nx = Nx;
	X.hmu = (T)(gp.dZ / 2.);
	X.sinv(ix, iy, X.rxx, X.ryy, X.rxy);
	X.va0 = X.vsum(0, ix, iy);
	X.va1 = X.vsum(1, ix, iy);
	const T dX = (T)gp.dX, dY = (T)gp.dY;
	auto ezz = [&](int x, int y) { int i = x + Nx * y; return (A[Q_IZZ * N + i] + B[Q_IZZ * N + i]) / (T)2; };
	T e0 = ezz(ix, iy);
	int pxq = (ix == Nx - 1) ? 1 : ix + 1, mxq = (ix == 0) ? Nx - 2 : ix - 1;
	int pyq = (iy == Ny - 1) ? 1 : iy + 1, myq = (iy == 0) ? Ny - 2 : iy - 1;
	int pxs = (ix == Nx - 2) ? 0 : ix + 1, mxs = (ix == 0) ? Nx - 2 : ix - 1;
	int pys = (iy == Ny - 2) ? 0 : iy + 1, mys = (iy == 0) ? Ny - 2 : iy - 1;
	cx<T> r[4];
	const cx<T> z = mk<T>(0, 0);

	// DX: rows ix < Nx-1 when Nx > 3; k = 0 mx, 1 centre, 2 px.
	{
		bool ok = Nx > 3 && ix < Nx - 1;
		T cm = 0, cp = 0, c0 = 0;
		if(ok) {
			cm = (T)0.5 * (ezz(mxq, iy) + e0) / (dX * dX);
			cp = (T)0.5 * (ezz(pxq, iy) + e0) / (dX * dX);
			c0 = -cm - cp;
		}
		const int cols[3] = {mxs, ix, pxs};
		const T c1[3] = {cm, c0, cp};
		const T L[3] = {(T)1 / (dX * dX), (T)-2 / (dX * dX), (T)1 / (dX * dX)};
		const T dd[3] = {(T)-0.5 / dX, 0, (T)0.5 / dX};
		for(int k = 0; k < 3; k++) {
			if(ok) {
				int cxp = cols[k];
				T kxx = X.avg(Q_XXTR, cxp, iy), kxy = X.avg(Q_XYTR, cxp, iy);
				X.entry(c1[k] * kxx, c1[k] * kxy, (T)0, L[k], cxp, iy, dd[k], 0, r);
			}
			else r[0] = r[1] = r[2] = r[3] = z;
			for(int b = 0; b < 4; b++) C[cidx(C_DX + 3 * b + k, p)] = cvt<S>(r[b]);
			Dg[(size_t)(0 * 6 + 0 * 3 + k) * N] = r[0];
			Dg[(size_t)(0 * 6 + 1 * 3 + k) * N] = r[3];
		}
	}
	// DY: rows iy < Ny-1 when Ny > 3; k = 0 my, 1 centre, 2 py.
	{
		bool ok = Ny > 3 && iy < Ny - 1;
		T cm = 0, cp = 0, c0 = 0;
		if(ok) {
			cp = (T)0.5 * (ezz(ix, pyq) + e0) / (dY * dY);
			cm = (T)0.5 * (ezz(ix, myq) + e0) / (dY * dY);
			c0 = -cm - cp;
		}
		const int rows[3] = {mys, iy, pys};
		const T c1[3] = {cm, c0, cp};
		const T L[3] = {(T)1 / (dY * dY), (T)-2 / (dY * dY), (T)1 / (dY * dY)};
		const T dd[3] = {(T)-0.5 / dY, 0, (T)0.5 / dY};
		for(int k = 0; k < 3; k++) {
			if(ok) {
				int cyp = rows[k];
				T kyy = X.avg(Q_YYTR, ix, cyp), kxy = X.avg(Q_XYTR, ix, cyp);
				X.entry(L[k], (T)0, c1[k] * kxy, c1[k] * kyy, ix, cyp, dd[k], 1, r);
			}
			else r[0] = r[1] = r[2] = r[3] = z;
			for(int b = 0; b < 4; b++) C[cidx(C_DY + 3 * b + k, p)] = cvt<S>(r[b]);
			Dg[(size_t)(1 * 6 + 0 * 3 + k) * N] = r[0];
			Dg[(size_t)(1 * 6 + 1 * 3 + k) * N] = r[3];
		}
	}
	// DXDY: rows ix < Nx-1, iy < Ny-1 when Nx > 3 and Ny > 3; k = pxpy, mxpy, pxmy, mxmy.
	{
		bool ok = Nx > 3 && Ny > 3 && ix < Nx - 1 && iy < Ny - 1;
		T a1 = 0, c1 = 0, a2 = 0, c2 = 0;
		const T q4 = (T)0.25;
		if(ok) {
			a1 = q4 * ezz(pxq, iy) / (dX * dY); c1 = q4 * ezz(mxq, iy) / (dX * dY);
			a2 = q4 * ezz(ix, pyq) / (dX * dY); c2 = q4 * ezz(ix, myq) / (dX * dY);
		}
		const T g0[4] = {-q4 / (dX * dY), q4 / (dX * dY), q4 / (dX * dY), -q4 / (dX * dY)};
		const T d01[4] = {a1, -c1, -a1, c1};
		const T d10[4] = {a2, -a2, -c2, c2};
		const int cxs[4] = {pxs, mxs, pxs, mxs};
		const int cys[4] = {pys, pys, mys, mys};
		for(int k = 0; k < 4; k++) {
			if(ok) {
				T kxx = X.avg(Q_XXTR, cxs[k], cys[k]), kyy = X.avg(Q_YYTR, cxs[k], cys[k]);
				T kxy = X.avg(Q_XYTR, cxs[k], cys[k]);
				X.entry(d01[k] * kxy, g0[k] + d01[k] * kyy, g0[k] + d10[k] * kxx, d10[k] * kxy,
					cxs[k], cys[k], (T)0, 0, r);
			}
			else r[0] = r[1] = r[2] = r[3] = z;
			for(int b = 0; b < 4; b++) C[cidx(C_DXDY + 4 * b + k, p)] = cvt<S>(r[b]);
		}
	}
}

// ---------------------------------------------------------------------------------------
// Right-hand-side kernels over all (point, slot) pairs of a pass.
// ---------------------------------------------------------------------------------------
template <typename R>
struct Stencil {
	const cx<R>* C;
	int N, Nx, Ny;
	__device__ __forceinline__ cx<R> c(int plane, int p) const { return C[cidx(plane, p)]; }
	// DX block b at row (x, y): columns mx, x, px with period Nx-1.
	__device__ __forceinline__ cx<R> dx(int b, int x, int y, const cx<R>* s) const {
		int p = x + Nx * y;
		int mx = x == 0 ? Nx - 2 : x - 1, px = x == Nx - 2 ? 0 : x + 1;
		int base = C_DX + 3 * b;
		return c(base, p) * s[mx + Nx * y] + c(base + 1, p) * s[p] + c(base + 2, p) * s[px + Nx * y];
	}
	__device__ __forceinline__ cx<R> dy(int b, int x, int y, const cx<R>* s) const {
		int p = x + Nx * y;
		int my = y == 0 ? Ny - 2 : y - 1, py = y == Ny - 2 ? 0 : y + 1;
		int base = C_DY + 3 * b;
		return c(base, p) * s[x + Nx * my] + c(base + 1, p) * s[p] + c(base + 2, p) * s[x + Nx * py];
	}
	__device__ __forceinline__ cx<R> dxdy(int b, int x, int y, const cx<R>* s) const {
		int p = x + Nx * y;
		int mx = x == 0 ? Nx - 2 : x - 1, px = x == Nx - 2 ? 0 : x + 1;
		int my = y == 0 ? Ny - 2 : y - 1, py = y == Ny - 2 ? 0 : y + 1;
		int base = C_DXDY + 4 * b;
		return c(base, p) * s[px + Nx * py] + c(base + 1, p) * s[mx + Nx * py] +
			c(base + 2, p) * s[px + Nx * my] + c(base + 3, p) * s[mx + Nx * my];
	}
	// Multi-slot forms: the same stencil coefficients applied to KS fields (slot planes
	// ss apart), accumulated into out[].
	template <int KS>
	__device__ __forceinline__ void dx_m(int b, int x, int y, const cx<R>* s, size_t ss, cx<R>* out) const {
		int p = x + Nx * y;
		int mx = x == 0 ? Nx - 2 : x - 1, px = x == Nx - 2 ? 0 : x + 1;
		int base = C_DX + 3 * b;
		cx<R> c0 = c(base, p), c1 = c(base + 1, p), c2 = c(base + 2, p);
#pragma unroll
		for(int j = 0; j < KS; j++) {
			const cx<R>* f = s + j * ss;
			out[j] = cfma(c2, f[px + Nx * y], cfma(c1, f[p], cfma(c0, f[mx + Nx * y], out[j])));
		}
	}
	template <int KS>
	__device__ __forceinline__ void dy_m(int b, int x, int y, const cx<R>* s, size_t ss, cx<R>* out) const {
		int p = x + Nx * y;
		int my = y == 0 ? Ny - 2 : y - 1, py = y == Ny - 2 ? 0 : y + 1;
		int base = C_DY + 3 * b;
		cx<R> c0 = c(base, p), c1 = c(base + 1, p), c2 = c(base + 2, p);
#pragma unroll
		for(int j = 0; j < KS; j++) {
			const cx<R>* f = s + j * ss;
			out[j] = cfma(c2, f[x + Nx * py], cfma(c1, f[p], cfma(c0, f[x + Nx * my], out[j])));
		}
	}
	template <int KS>
	__device__ __forceinline__ void dxdy_m(int b, int x, int y, const cx<R>* s, size_t ss, cx<R>* out) const {
		int p = x + Nx * y;
		int mx = x == 0 ? Nx - 2 : x - 1, px = x == Nx - 2 ? 0 : x + 1;
		int my = y == 0 ? Ny - 2 : y - 1, py = y == Ny - 2 ? 0 : y + 1;
		int base = C_DXDY + 4 * b;
		cx<R> c0 = c(base, p), c1 = c(base + 1, p), c2 = c(base + 2, p), c3 = c(base + 3, p);
#pragma unroll
		for(int j = 0; j < KS; j++) {
			const cx<R>* f = s + j * ss;
			out[j] = cfma(c3, f[mx + Nx * my], cfma(c2, f[px + Nx * my], cfma(c1, f[mx + Nx * py], cfma(c0, f[px + Nx * py], out[j]))));
		}
	}
};

// Step kinds of the composite stencil kernel (ParaxialPrimaryEvolutionOperator.cpp:153-207
// with the duplicate-row/column fix-ups of BlockSparseMatrix.cpp folded in analytically).
enum { ST_EXPL_Y = 0, ST_EXPL_X = 1, ST_WOOD_X = 2, ST_WOOD_Y = 3 };

// One component of a composite stencil step at point (ix, iy). EXPL kinds return
// f + mu*R f (explicit half-step), WOOD kinds return mu*R_offdiag t (Woodbury right-hand side).
// (xx, yy) are the indices with the duplicate column / row folded onto column / row 0, which
// is where the reference's fix-ups copy their values from.
template <typename R, int KIND>
__device__ __forceinline__ cx<R> composite(const Stencil<R>& st, int comp, int ix, int iy,
		const cx<R>* f0, const cx<R>* f1) {
	const int Nx = st.Nx, Ny = st.Ny;
	const int xx = ix == Nx - 1 ? 0 : ix, yy = iy == Ny - 1 ? 0 : iy;
	const bool ax = Nx > 3, ay = Ny > 3;
	cx<R> T = mk<R>(0, 0);
	if(KIND == ST_EXPL_Y) {
		if(comp == 0) {
			if(ay) T = st.dy(0, ix, yy, f0) + st.dy(1, ix, yy, f1);
			return f0[ix + Nx * iy] + T;
		}
		if(ay) {
			if(ax) T = st.dy(3, xx, yy, f1) + st.dxdy(3, xx, yy, f1) + st.dy(2, xx, yy, f0) + st.dxdy(2, xx, yy, f0);
			else T = st.dy(3, ix, yy, f1) + st.dy(2, ix, yy, f0);
		}
		return f1[ix + Nx * iy] + T;
	}
	if(KIND == ST_EXPL_X) {
		if(comp == 0) {
			if(ax) {
				if(ay) T = st.dx(0, xx, yy, f0) + st.dxdy(0, xx, yy, f0) + st.dx(1, xx, yy, f1) + st.dxdy(1, xx, yy, f1);
				else T = st.dx(0, xx, iy, f0) + st.dx(1, xx, iy, f1);
			}
			return f0[ix + Nx * iy] + T;
		}
		if(ax) T = st.dx(3, xx, iy, f1) + st.dx(2, xx, iy, f0);
		return f1[ix + Nx * iy] + T;
	}
	if(KIND == ST_WOOD_X) {
		if(comp == 0) {
			if(ax) {
				if(ay) T = st.dx(1, xx, yy, f1) + st.dxdy(1, xx, yy, f1) + st.dxdy(0, xx, yy, f0);
				else T = st.dx(1, xx, iy, f1);
			}
			return T;
		}
		if(ax) T = st.dx(2, xx, iy, f0);
		return T;
	}
	// ST_WOOD_Y
	if(comp == 0) {
		if(ay) T = st.dy(1, ix, yy, f1);
		return T;
	}
	if(ay) {
		if(ax) T = st.dy(2, xx, yy, f0) + st.dxdy(2, xx, yy, f0) + st.dxdy(3, xx, yy, f1);
		else T = st.dy(2, ix, yy, f0);
	}
	return T;
}

// composite() for KS consecutive slots at once (f0: comp-0 plane of the first slot, slot
// planes 2N apart, comp-1 plane at +N); every stencil coefficient is loaded once.
template <typename R, int KIND, int KS>
__device__ __forceinline__ void composite_m(const Stencil<R>& st, int comp, int ix, int iy, const cx<R>* f0,
		cx<R>* out) {
	const int Nx = st.Nx, Ny = st.Ny;
	const size_t N = st.N, ss = 2 * N;
	const cx<R>* f1 = f0 + N;
	const int xx = ix == Nx - 1 ? 0 : ix, yy = iy == Ny - 1 ? 0 : iy;
	const bool ax = Nx > 3, ay = Ny > 3;
	const int p = ix + Nx * iy;
#pragma unroll
	for(int j = 0; j < KS; j++) out[j] = mk<R>(0, 0);
	if(KIND == ST_EXPL_Y) {
		if(comp == 0) {
			if(ay) { st.template dy_m<KS>(0, ix, yy, f0, ss, out); st.template dy_m<KS>(1, ix, yy, f1, ss, out); }
#pragma unroll
			for(int j = 0; j < KS; j++) out[j] += f0[j * ss + p];
			return;
		}
		if(ay) {
			if(ax) {
				st.template dy_m<KS>(3, xx, yy, f1, ss, out); st.template dxdy_m<KS>(3, xx, yy, f1, ss, out);
				st.template dy_m<KS>(2, xx, yy, f0, ss, out); st.template dxdy_m<KS>(2, xx, yy, f0, ss, out);
			}
			else { st.template dy_m<KS>(3, ix, yy, f1, ss, out); st.template dy_m<KS>(2, ix, yy, f0, ss, out); }
		}
#pragma unroll
		for(int j = 0; j < KS; j++) out[j] += f1[j * ss + p];
		return;
	}
	if(KIND == ST_EXPL_X) {
		if(comp == 0) {
			if(ax) {
				if(ay) {
					st.template dx_m<KS>(0, xx, yy, f0, ss, out); st.template dxdy_m<KS>(0, xx, yy, f0, ss, out);
					st.template dx_m<KS>(1, xx, yy, f1, ss, out); st.template dxdy_m<KS>(1, xx, yy, f1, ss, out);
				}
				else { st.template dx_m<KS>(0, xx, iy, f0, ss, out); st.template dx_m<KS>(1, xx, iy, f1, ss, out); }
			}
#pragma unroll
			for(int j = 0; j < KS; j++) out[j] += f0[j * ss + p];
			return;
		}
		if(ax) { st.template dx_m<KS>(3, xx, iy, f1, ss, out); st.template dx_m<KS>(2, xx, iy, f0, ss, out); }
#pragma unroll
		for(int j = 0; j < KS; j++) out[j] += f1[j * ss + p];
		return;
	}
	if(KIND == ST_WOOD_X) {
		if(comp == 0) {
			if(ax) {
				if(ay) {
					st.template dx_m<KS>(1, xx, yy, f1, ss, out); st.template dxdy_m<KS>(1, xx, yy, f1, ss, out);
					st.template dxdy_m<KS>(0, xx, yy, f0, ss, out);
				}
				else st.template dx_m<KS>(1, xx, iy, f1, ss, out);
			}
			return;
		}
		if(ax) st.template dx_m<KS>(2, xx, iy, f0, ss, out);
		return;
	}
	if(comp == 0) {
		if(ay) st.template dy_m<KS>(1, ix, yy, f1, ss, out);
		return;
	}
	if(ay) {
		if(ax) {
			st.template dy_m<KS>(2, xx, yy, f0, ss, out); st.template dxdy_m<KS>(2, xx, yy, f0, ss, out);
			st.template dxdy_m<KS>(3, xx, yy, f1, ss, out);
		}
		else st.template dy_m<KS>(2, ix, yy, f0, ss, out);
	}
}

template <typename R, int KIND>
__global__ void k_stencil(Geom G, int slot0, const cx<R>* __restrict__ coef, const cx<R>* __restrict__ src,
		cx<R>* __restrict__ dst) {
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	int N = G.N, Nx = G.Nx, Ny = G.Ny;
	if(p >= N) return;
	int s = blockIdx.y;
	int g = (slot0 + s) / G.spg - slot0 / G.spg;
	Stencil<R> st{coef + (size_t)g * coef_set_size(N), N, Nx, Ny};
	const cx<R>* f0 = src + (size_t)s * 2 * N;
	const cx<R>* f1 = f0 + N;
	int ix = p % Nx, iy = p / Nx;
	dst[(size_t)s * 2 * N + p] = composite<R, KIND>(st, 0, ix, iy, f0, f1);
	dst[(size_t)s * 2 * N + N + p] = composite<R, KIND>(st, 1, ix, iy, f0, f1);
}

// Periodic line solve with the pre-factored Thomas/Sherman-Morrison data, sequential form:
// one thread per (line, comp, slot). Used for lines too long for the chunked kernels.
// dst may alias src. If acc_out is set: acc_out = acc_in + x.
template <typename R, int DIRN>
__global__ void k_solve(Geom G, int slot0, int nslots, const cx<R>* __restrict__ fac, size_t plane,
		const cx<double>* __restrict__ lsc, const cx<R>* src, cx<R>* dst,
		const cx<R>* acc_in, cx<R>* acc_out) {
	int Nx = G.Nx, Ny = G.Ny, N = G.N;
	int L = DIRN == 0 ? Nx : Ny;
	int nlines = DIRN == 0 ? Ny : Nx;
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if(t >= nslots * 2 * nlines) return;
	int line = t % nlines;
	int c = (t / nlines) % 2;
	int s = t / (2 * nlines);
	int g = (slot0 + s) / G.spg - slot0 / G.spg;
	size_t off = (size_t)s * 2 * N + (size_t)c * N;
	const cx<R>* S = src + off;
	cx<R>* D = dst + off;
	const int stride = DIRN == 0 ? 1 : Nx;
	const int base = DIRN == 0 ? Nx * line : line;
	if(L <= 3) {
		for(int i = 0; i < L; i++) {
			int q = base + i * stride;
			cx<R> x = S[q];
			D[q] = x;
			if(acc_out) acc_out[off + q] = acc_in[off + q] + x;
		}
		return;
	}
	const cx<R>* Fc = fac + ((size_t)g * 2 + c) * NFAC * plane;
	const cx<double>* ls = lsc + (((size_t)g * 2 + c) * nlines + line) * 2;
	int q = base;
	cx<R> d = S[q] * Fc[F_RB * plane + q];
	cx<R> acc = d;
	D[q] = d;
	for(int i = 1; i < L - 1; i++) {
		q += stride;
		d = Fc[F_A * plane + q] * d + S[q] * Fc[F_RB * plane + q];
		acc += Fc[F_W * plane + q] * d;
		D[q] = d;
	}
	cx<double> frac = (cvt<double>(acc) - ls[0] * cvt<double>(d)) * ls[1];
	cx<R> fr = cvt<R>(frac);
	cx<R> dn = d;
	cx<R> x = dn - fr * Fc[F_COR * plane + q];
	D[q] = x;
	if(acc_out) acc_out[off + q] = acc_in[off + q] + x;
	for(int i = L - 2; i > 0; i--) {
		q -= stride;
		cx<R> dp = D[q] + Fc[F_C * plane + q] * dn;
		x = dp - fr * Fc[F_COR * plane + q];
		D[q] = x;
		if(acc_out) acc_out[off + q] = acc_in[off + q] + x;
		dn = dp;
	}
	int qe = base + (L - 1) * stride;
	D[qe] = x;  // duplicate point = x_0
	if(acc_out) acc_out[off + qe] = acc_in[off + qe] + x;
}

template <typename R>
__device__ __forceinline__ cx<R> shfl_up_c(cx<R> v, int d) {
	return mk<R>(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}
template <typename R>
__device__ __forceinline__ cx<R> shfl_down_c(cx<R> v, int d) {
	return mk<R>(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
}
template <typename R>
__device__ __forceinline__ cx<R> shfl_idx_c(cx<R> v, int l) {
	return mk<R>(__shfl_sync(0xffffffffu, v.x, l), __shfl_sync(0xffffffffu, v.y, l));
}
template <typename R>
__device__ __forceinline__ cx<R> shfl_xor_c(cx<R> v, int m) {
	return mk<R>(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// x-line solve fused with the right-hand side that precedes it (KIND: explicit y half-step or
// x Woodbury term), chunked parallel form: one warp per (line, comp, KS slots of one
// wavelength); lane l owns the unknowns [l*M, l*M+M) of the line. The forward and backward
// recurrences are composed per chunk, combined by warp-shuffle scans and replayed, so every
// sweep is parallel over 32 lanes. The right-hand side is formed with each stencil
// coefficient loaded once for the KS slots and staged through shared memory so that global
// accesses stay coalesced; the factor planes are stored chunk-interleaved (element l*M+k at
// k*32+l) and are also loaded once for the KS slots. Block = LT warps = LT lines.
// ---------------------------------------------------------------------------------------
// The y-line solves as x-line solves of the transposed frame (x' = y, y' = x, components
// exchanged): the stencil blocks b become 3 - b (00 <-> 11, 01 <-> 10), the DX and DY stencils
// exchange, the DXDY corners (px,py), (mx,py), (px,my), (mx,my) become corners 0, 2, 1, 3, and the
// duplicate-row/column folding and the period-(N-1) wraps map onto themselves. This kernel
// writes, per wavelength group, the transposed planes those solves read: DY' (every block) from
// DX, DX' (blocks 1 and 2) from DY, every DXDY' block from DXDY, and the diagonal stencils of the
// transposed x-lines (diag' direction 0, component c') from the y diagonals of component 1 - c'.
// Each block moves one 32x32 tile of one plane through shared memory (coalesced reads and writes).
constexpr int NCT = 12 + 6 + 16 + 6;  // planes per group: DY', DX' (blocks 1, 2), DXDY', diag'
template <typename S>
__global__ void __launch_bounds__(256) k_coef_t(Geom G, const cx<S>* __restrict__ coef, const cx<S>* __restrict__ diag,
		cx<S>* __restrict__ coefT, cx<S>* __restrict__ diagT) {
	__shared__ cx<S> tile[32][33];
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int g = blockIdx.z / NCT, k = blockIdx.z % NCT;
	int sp, dp;  // source / destination plane
	bool dg = false;
	if(k < 12) { const int b = k / 3, kk = k % 3; dp = C_DY + 3 * b + kk; sp = C_DX + 3 * (3 - b) + kk; }
	else if(k < 18) { const int b = 1 + (k - 12) / 3, kk = (k - 12) % 3; dp = C_DX + 3 * b + kk; sp = C_DY + 3 * (3 - b) + kk; }
	else if(k < 34) {
		const int b = (k - 18) / 4, kk = (k - 18) % 4;
		const int sk = kk == 1 ? 2 : kk == 2 ? 1 : kk;
		dp = C_DXDY + 4 * b + kk; sp = C_DXDY + 4 * (3 - b) + sk;
	}
	else { const int cp = (k - 34) / 3, kk = (k - 34) % 3; dp = 0 * 6 + cp * 3 + kk; sp = 1 * 6 + (1 - cp) * 3 + kk; dg = true; }
	// diagonal stencils: plain planes; coefficient planes: the tiled layout (cidx)
	const cx<S>* src = dg ? diag + (size_t)g * NDIAG * N : coef + (size_t)g * coef_set_size(N);
	cx<S>* dst = dg ? diagT + (size_t)g * NDIAG * N : coefT + (size_t)g * coef_set_size(N);
	auto at = [&](int plane, int q) { return dg ? (size_t)plane * N + q : cidx(plane, q); };
	const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
	for(int r = threadIdx.y; r < 32; r += blockDim.y) {
		const int x = x0 + threadIdx.x, y = y0 + r;
		if(x < Nx && y < Ny) tile[r][threadIdx.x] = src[at(sp, y * Nx + x)];
	}
	__syncthreads();
	for(int r = threadIdx.y; r < 32; r += blockDim.y) {
		const int y = y0 + threadIdx.x, x = x0 + r;  // destination row x, column y
		if(x < Nx && y < Ny) dst[at(dp, x * Ny + y)] = tile[threadIdx.x][r];
	}
}

// Pre-factorisation of the periodic line solves (I - mu*R_cc) x = b per (group, comp, line), in
// the plan's precision. Restates shifted_block_vmult_inv (BlockSparseMatrix.cpp:195-258 and
// 386-449): Thomas sweep with beta0 = 2*mid0 and the Sherman-Morrison corner vector corr
// (corr0 = -1/2). Everything that does not depend on the right-hand side is computed here once
// per (wavelength, slab) and shared by all (q, pol) slots:
//   F_A    alpha_i = -inf_i/beta_i   F_RB  1/beta_i        F_C   -gamma_i
//   F_COR  corr_i after back-substitution
//   F_W    w_i = prod_{j<i}(-gamma_j), so that the back-substituted x_0 = sum_i w_i d_i
//          is formed during the forward sweep
// plus per line r0 = inf0/mid0 and rden = 1/(1 + corr0 - r0*corr_{L-2}) in FP64. The forward
// sweep of a solve is then d_i = alpha_i d_{i-1} + b_i/beta_i and the backward sweep
// x_{i-1} = d_{i-1} - gamma_{i-1} x_i: both first-order affine recurrences whose coefficients
// do not depend on b, which is what the chunked solves exploit.
// Chunk-parallel form: every line is split into chunks processed by different threads. The
// pivots follow the continued fraction
// beta_i = mid'_i - inf_i sup_{i-1} / beta_{i-1}, a Moebius map: (p, q) -> M_i (p, q) with
// M_i = [[mid'_i, -inf_i sup_{i-1}], [1, 0]] and beta = p / q. Each chunk forms the product of
// its maps (rescaled to keep it bounded; the map is projective), the chunk products are
// combined with an exclusive scan, and each chunk replays its elements from the pivot before
// it. corr (forward), the back-substituted corr and w are affine recurrences combined the same
// way. x-lines: one warp per line, lanes = chunks of chunkM elements (the interleaved factor
// layout), combined with shuffles. y-lines: 32 columns per block (lanes), warps = chunks of
// rows, combined through shared memory. Intermediate values go to the output planes and are
// read back by the same thread.
template <typename T>
struct Mob {
	cx<T> a, b, c, d;  // [[a, b], [c, d]]
};
template <typename T>
__device__ __forceinline__ Mob<T> mob_mul(const Mob<T>& X, const Mob<T>& Y) {  // X . Y
	return Mob<T>{X.a * Y.a + X.b * Y.c, X.a * Y.b + X.b * Y.d, X.c * Y.a + X.d * Y.c, X.c * Y.b + X.d * Y.d};
}
template <typename T>
__device__ __forceinline__ T l1abs(cx<T> z) { return fabs(z.x) + fabs(z.y); }
template <typename T>
__device__ __forceinline__ void mob_norm(Mob<T>& X) {
	T m = fmax(fmax(l1abs(X.a), l1abs(X.b)), fmax(l1abs(X.c), l1abs(X.d)));
	if(m > (T)0) {
		T r = (T)1 / m;
		X.a = X.a * r; X.b = X.b * r; X.c = X.c * r; X.d = X.d * r;
	}
}
template <typename T>
struct Aff {
	cx<T> A, B;  // x -> A x + B
};
template <typename T>
__device__ __forceinline__ Aff<T> aff_after(const Aff<T>& second, const Aff<T>& first) {
	return Aff<T>{second.A * first.A, second.A * first.B + second.B};
}
template <typename T>
__device__ __forceinline__ Mob<T> shfl_up_m(const Mob<T>& X, int o) {
	return Mob<T>{shfl_up_c(X.a, o), shfl_up_c(X.b, o), shfl_up_c(X.c, o), shfl_up_c(X.d, o)};
}
template <typename T>
__device__ __forceinline__ Aff<T> shfl_up_a(const Aff<T>& X, int o) { return Aff<T>{shfl_up_c(X.A, o), shfl_up_c(X.B, o)}; }
template <typename T>
__device__ __forceinline__ Aff<T> shfl_down_a(const Aff<T>& X, int o) { return Aff<T>{shfl_down_c(X.A, o), shfl_down_c(X.B, o)}; }

template <typename S, int DIRN>
__global__ void __launch_bounds__(DIRN == 1 ? 512 : 256) k_factor_chunked(Geom G, int ngroups, int chunkMx, int chunksX, int W,
		const cx<S>* __restrict__ diag, cx<S>* __restrict__ fac, size_t plane, cx<double>* __restrict__ lsc) {
	typedef S T;
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int L = DIRN == 0 ? Nx : Ny;
	const int nlines = DIRN == 0 ? Ny : Nx;
	const int n = L - 1;
	const int lane = threadIdx.x, w = threadIdx.y;
	int line, gc, chunk, nchunks, M;
	if(DIRN == 0) {
		line = blockIdx.x * blockDim.y + w;
		gc = blockIdx.y;
		chunk = lane;
		nchunks = 32;
		M = (n + 31) / 32;
	}
	else {
		line = blockIdx.x * 32 + lane;
		gc = blockIdx.y;
		chunk = w;
		nchunks = W;
		M = (n + W - 1) / W;
	}
	const bool active = line < nlines && L > 3;
	const int g = gc / 2, c = gc % 2;
	const int i0 = chunk * M, i1 = min(i0 + M, n);
	const cx<T>* Dg = diag + (size_t)g * NDIAG * N + (size_t)(DIRN * 6 + c * 3) * N;
	cx<S>* Fc = fac + ((size_t)g * 2 + c) * NFAC * plane;
	const int stride = DIRN == 0 ? 1 : Nx;
	const int base = DIRN == 0 ? Nx * line : line;
	auto P = [&](int i) { return base + i * stride; };
	// storage of factor f of element i: natural layout (plane f, point P(i)), or the solves'
	// chunk-interleaved x layout: chunksX chunks of chunkMx elements per line, element
	// i = ci*chunkMx + k of factor f at ((line*chunkMx + k)*NFAC + f)*chunksX + ci, so that the
	// factors a lane reads for one element are compile-time offsets from one address
	auto Q = [&](int f, int i) -> size_t {
		if(DIRN == 1 || chunkMx <= 0) return (size_t)f * plane + P(i);
		return (((size_t)line * chunkMx + i % chunkMx) * NFAC + f) * chunksX + (i / chunkMx);
	};
	const cx<T> one = mk<T>(1, 0), zero = mk<T>(0, 0);
	auto sup = [&](int i) { return -Dg[2 * (size_t)N + P(i)]; };
	auto mid = [&](int i) { return one - Dg[1 * (size_t)N + P(i)]; };
	auto inf = [&](int i) { return -Dg[P(i)]; };
	cx<T> m0 = zero, a0 = zero, corner = zero;
	if(active) {
		m0 = mid(0);
		a0 = inf(0);
		corner = cdiv(sup(n - 1) * a0, m0);
	}
	auto midp = [&](int i) { return i == n - 1 ? mid(i) + corner : mid(i); };
	// shared memory for the y combine: [W][32] per quantity
	extern __shared__ unsigned char smem_raw[];
	Mob<T>* shM = reinterpret_cast<Mob<T>*>(smem_raw);
	Aff<T>* shA = reinterpret_cast<Aff<T>*>(shM + (DIRN == 1 ? W * 32 : 0));
	Aff<T>* shB = shA + (DIRN == 1 ? W * 32 : 0);
	cx<T>* shX = reinterpret_cast<cx<T>*>(shB + (DIRN == 1 ? W * 32 : 0));  // [2][32] corr_last, cv0

	// ---- 1. pivots: chunk product of the Moebius maps ----
	Mob<T> Pm{one, zero, zero, one};
	if(active) {
		for(int i = i0; i < i1; i++) {
			Mob<T> Mi;
			if(i == 0) Mi = Mob<T>{zero, (T)2 * m0, zero, one};
			else Mi = Mob<T>{midp(i), -(inf(i) * sup(i - 1)), one, zero};
			Pm = mob_mul(Mi, Pm);
			mob_norm(Pm);
		}
	}
	// exclusive scan over chunks in order: Sx = P_{c-1} ... P_0
	Mob<T> Sx{one, zero, zero, one};
	if(DIRN == 0) {
		Mob<T> X = Pm;
#pragma unroll
		for(int o = 1; o < 32; o <<= 1) {
			Mob<T> Y = shfl_up_m(X, o);
			if(lane >= o) { X = mob_mul(X, Y); mob_norm(X); }
		}
		Mob<T> E = shfl_up_m(X, 1);
		if(lane > 0) Sx = E;
	}
	else {
		shM[w * 32 + lane] = Pm;
		__syncthreads();
		if(w == 0) {
			Mob<T> acc{one, zero, zero, one};
			for(int k = 0; k < W; k++) {
				Mob<T> pk = shM[k * 32 + lane];
				shM[k * 32 + lane] = acc;
				acc = mob_mul(pk, acc);
				mob_norm(acc);
			}
		}
		__syncthreads();
		Sx = shM[w * 32 + lane];
	}
	// replay: beta, and the chunk maps of corr (forward) and w
	// (the divisions by the previous pivot are multiplications by its reciprocal, computed one step
	// earlier)
	Aff<T> Fcorr{one, zero}, Fw{one, zero};
	cx<T> rb_prev = zero;
	if(active && i0 < i1) {
		if(i0 > 0) rb_prev = crecip(cdiv(Sx.b, Sx.d));  // state before the chunk: Sx . (0, 1)
		for(int i = i0; i < i1; i++) {
			cx<T> beta = i == 0 ? (T)2 * m0 : midp(i) - (inf(i) * sup(i - 1)) * rb_prev;
			cx<T> rb = crecip(beta);
			cx<T> alpha = i == 0 ? zero : -(inf(i) * rb);
			Fc[Q(F_RB, i)] = cvt<S>(rb);
			Fc[Q(F_A, i)] = cvt<S>(alpha);
			Fc[Q(F_C, i)] = i < n - 1 ? cvt<S>(-(sup(i) * rb)) : mk<S>(0, 0);
			// corr_0 = -1/2, corr_i = alpha_i corr_{i-1} (+ sup_{n-1} rb_{n-1} on the last row)
			Aff<T> ec = i == 0 ? Aff<T>{zero, mk<T>(-0.5, 0)} : Aff<T>{alpha, i == n - 1 ? sup(i) * rb : zero};
			Fcorr = aff_after(ec, Fcorr);
			// w_0 = 1, w_i = -gamma_{i-1} w_{i-1}, gamma_{i-1} = sup_{i-1} / beta_{i-1}
			Aff<T> ew = i == 0 ? Aff<T>{zero, one} : Aff<T>{-(sup(i - 1) * rb_prev), zero};
			Fw = aff_after(ew, Fw);
			rb_prev = rb;
		}
	}
	// ---- 2. exclusive scans of the corr and w maps, replay ----
	Aff<T> Ec{one, zero}, Ew{one, zero};
	if(DIRN == 0) {
		Aff<T> Xc = Fcorr, Xw = Fw;
#pragma unroll
		for(int o = 1; o < 32; o <<= 1) {
			Aff<T> Yc = shfl_up_a(Xc, o), Yw = shfl_up_a(Xw, o);
			if(lane >= o) { Xc = aff_after(Xc, Yc); Xw = aff_after(Xw, Yw); }
		}
		Aff<T> Pc = shfl_up_a(Xc, 1), Pw = shfl_up_a(Xw, 1);
		if(lane > 0) { Ec = Pc; Ew = Pw; }
	}
	else {
		__syncthreads();
		shA[w * 32 + lane] = Fcorr;
		shB[w * 32 + lane] = Fw;
		__syncthreads();
		if(w == 0) {
			Aff<T> ac{one, zero}, aw{one, zero};
			for(int k = 0; k < W; k++) {
				Aff<T> fc = shA[k * 32 + lane], fw = shB[k * 32 + lane];
				shA[k * 32 + lane] = ac;
				shB[k * 32 + lane] = aw;
				ac = aff_after(fc, ac);
				aw = aff_after(fw, aw);
			}
		}
		__syncthreads();
		Ec = shA[w * 32 + lane];
		Ew = shB[w * 32 + lane];
	}
	if(DIRN == 0) __syncwarp();  // F_C of the previous chunk, written by another lane
	cx<T> corr_last = zero;
	bool own_last = active && i0 <= n - 1 && n - 1 < i1;
	if(active && i0 < i1) {
		cx<T> cr = Ec.B, wv = Ew.B;  // values before the chunk (maps applied to 0)
		for(int i = i0; i < i1; i++) {
			cx<T> alpha = cvt<T>(Fc[Q(F_A, i)]);
			cx<T> rb = cvt<T>(Fc[Q(F_RB, i)]);
			if(i == 0) { cr = mk<T>(-0.5, 0); wv = one; }
			else {
				cx<T> gm = -cvt<T>(Fc[Q(F_C, i - 1)]);  // gamma_{i-1}
				cr = cfma(alpha, cr, (i == n - 1 ? sup(i) * rb : zero));
				wv = -(gm * wv);
			}
			Fc[Q(F_COR, i)] = cvt<S>(cr);  // forward corr, replaced below
			Fc[Q(F_W, i)] = cvt<S>(wv);
			if(i == n - 1) corr_last = cr;
		}
	}
	// broadcast corr_last to the line
	if(DIRN == 0) {
		corr_last = shfl_idx_c(corr_last, (n - 1) / M);
	}
	else {
		__syncthreads();
		if(own_last) shX[lane] = corr_last;
		__syncthreads();
		corr_last = shX[lane];
	}
	// ---- 3. back-substituted corr: cv_{n-1} = corr_last, cv_j = -gamma_j cv_{j+1} + corr_j ----
	Aff<T> Bm{one, zero};
	if(active && i0 < i1) {
		for(int j = i1 - 1; j >= i0; j--) {
			Aff<T> e = j == n - 1 ? Aff<T>{zero, corr_last}
				: Aff<T>{cvt<T>(Fc[Q(F_C, j)]), cvt<T>(Fc[Q(F_COR, j)])};
			Bm = aff_after(e, Bm);
		}
	}
	Aff<T> Eb{one, zero};
	if(DIRN == 0) {
		Aff<T> X = Bm;
#pragma unroll
		for(int o = 1; o < 32; o <<= 1) {
			Aff<T> Y = shfl_down_a(X, o);
			if(lane + o < 32) X = aff_after(X, Y);
		}
		Aff<T> Nn = shfl_down_a(X, 1);
		if(lane < 31) Eb = Nn;
	}
	else {
		__syncthreads();
		shA[w * 32 + lane] = Bm;
		__syncthreads();
		if(w == 0) {
			Aff<T> acc{one, zero};
			for(int k = W - 1; k >= 0; k--) {
				Aff<T> f = shA[k * 32 + lane];
				shA[k * 32 + lane] = acc;
				acc = aff_after(f, acc);
			}
		}
		__syncthreads();
		Eb = shA[w * 32 + lane];
	}
	cx<T> cv0 = zero;
	if(active && i0 < i1) {
		cx<T> cv = Eb.B;  // cv of the element after the chunk
		for(int j = i1 - 1; j >= i0; j--) {
			cv = j == n - 1 ? corr_last
				: cvt<T>(Fc[Q(F_C, j)]) * cv + cvt<T>(Fc[Q(F_COR, j)]);
			Fc[Q(F_COR, j)] = cvt<S>(cv);
		}
		if(i0 == 0) cv0 = cv;
	}
	// padding of the interleaved x layout: identity maps
	if(DIRN == 0 && chunkMx > 0 && active) {
		for(int i = n + lane; i < chunksX * chunkMx; i += 32) {
			Fc[Q(F_A, i)] = mk<S>(0, 0);
			Fc[Q(F_RB, i)] = mk<S>(0, 0);
			Fc[Q(F_W, i)] = mk<S>(0, 0);
			Fc[Q(F_C, i)] = mk<S>(0, 0);
			Fc[Q(F_COR, i)] = mk<S>(0, 0);
		}
	}
	// Sherman-Morrison scalars in FP64
	if(active && chunk == 0) {
		cx<double>* ls = lsc + (((size_t)g * 2 + c) * nlines + line) * 2;
		cx<double> r0 = cdiv(cvt<double>(a0), cvt<double>(m0));
		ls[0] = r0;
		ls[1] = crecip(mk(1.0, 0.0) + cvt<double>(cv0) - r0 * cvt<double>(corr_last));
	}
}

// One combine of the chunk maps of a line whose chunks sit on the 32 lanes of a warp (chunk =
// lane; lanes past the line carry identity maps). Inputs per lane: forward map (P, d0[j]),
// sum terms (S0[j], S1), backward terms (Cp, G0[j], G1). Outputs per lane: din = the forward
// value entering the chunk, xin = the backward value entering it from the line's end, and
// fr = (sum_i w_i d_i - r0 * d_last) * rden, the Sherman-Morrison factor (same on all lanes).
template <typename R, int KS>
__device__ __forceinline__ void line_combine(cx<R> P, const cx<R>* d0, const cx<R>* S0, cx<R> S1, const cx<R>* G0,
		cx<R> G1, cx<R> Cp, cx<double> r0, cx<double> rden, int lane, cx<R>* din, cx<R>* xin, cx<R>* fr) {
	const cx<R> zero = mk<R>(0, 0);
	cx<R> B[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) B[j] = d0[j];
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
		const cx<R> Pp = shfl_up_c(P, o);
#pragma unroll
		for(int j = 0; j < KS; j++) {
			const cx<R> Bp = shfl_up_c(B[j], o);
			if(lane >= o) B[j] = cfma(P, Bp, B[j]);
		}
		if(lane >= o) P = P * Pp;
	}
	cx<R> G[KS];
	cx<R> tsel = zero, dsel = zero;  // lane j < KS keeps slot j's sum and last value
#pragma unroll
	for(int j = 0; j < KS; j++) {
		din[j] = shfl_up_c(B[j], 1);
		if(lane == 0) din[j] = zero;
		cx<R> t = cfma(S1, din[j], S0[j]);
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) t += shfl_xor_c(t, o);
		const cx<R> dl = shfl_idx_c(B[j], 31);
		if(lane == j) { tsel = t; dsel = dl; }
		G[j] = cfma(G1, din[j], G0[j]);
	}
	// the FP64 factor once per slot (lane j), then broadcast
	cx<R> f = zero;
	if(lane < KS) f = cvt<R>((cvt<double>(tsel) - r0 * cvt<double>(dsel)) * rden);
#pragma unroll
	for(int j = 0; j < KS; j++) fr[j] = shfl_idx_c(f, j);
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
		const cx<R> Cn = shfl_down_c(Cp, o);
#pragma unroll
		for(int j = 0; j < KS; j++) {
			const cx<R> Gn = shfl_down_c(G[j], o);
			if(lane + o < 32) G[j] = cfma(Cp, Gn, G[j]);
		}
		if(lane + o < 32) Cp = Cp * Cn;
	}
#pragma unroll
	for(int j = 0; j < KS; j++) {
		xin[j] = shfl_down_c(G[j], 1);
		if(lane == 31) xin[j] = zero;
	}
}

// x-line solve fused with its right-hand side (KIND: explicit y half-step or x Woodbury term):
// a warp per line (4 lines per block) for KS slots of one wavelength. The right-hand sides are
// computed with coalesced loads into the warp's shared buffer in the lane-chunk layout (lane l
// holds points [l M, l M + M)), one pass builds the chunk maps, line_combine joins them by
// shuffles, and a last pass finishes the line, which goes back out coalesced.
template <typename R, int M, int KIND, int KS, bool TOUT = false>
// Resident blocks per SM requested from the compiler: 8 (64 registers) for the instances
// whose chunk values fit, measured faster on GB300; the larger instances keep their registers.
#ifndef NBPM_XC_MINB
#define NBPM_XC_MINB(MK) ((MK) <= 16 ? 8 : 1)
#endif
#ifndef NBPM_YC_MINB
#define NBPM_YC_MINB 1
#endif
// TOUT: the results go out transposed with the two components exchanged ((c, iy, e) -> (1 - c,
// e, iy) of an Ny x Nx plane), written by the whole block so that each (point, LT lines) group
// is one 32-byte segment: the hand-over between the x-line frame and the transposed frame in
// which the y-lines are solved as x-lines (ADI with transposed y solves).
__global__ void __launch_bounds__(128, NBPM_XC_MINB(M * KS)) k_solve_xc(Geom G, int slot0, int nch, const cx<R>* __restrict__ coef,
		const cx<R>* __restrict__ fac, size_t plane, const cx<double>* __restrict__ lsc,
		const cx<R>* __restrict__ src, cx<R>* __restrict__ dst, const cx<R>* acc_in, cx<R>* acc_out,
		const cx<R>* acc_in2) {
	extern __shared__ unsigned char smem_raw[];
	constexpr int LT = 4;  // lines (warps) per block: launched with 128 threads
	const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int iy = blockIdx.x * LT + warp;
	if(!TOUT && iy >= Ny) return;
	const int c = blockIdx.y % 2, bc = blockIdx.y / 2;
	const int g = bc / nch, ch = bc % nch;
	const int s0 = g * G.spg + ch * KS;  // first slot (pass-relative)
	const int n_unk = Nx - 1;
	const int PITCH = 32 * (M + 1);
	cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw) + (size_t)warp * KS * PITCH;
	if(iy < Ny) {  // always true unless TOUT (whose block writes together after a barrier)
	const cx<R>* Fc = fac + ((size_t)g * 2 + c) * NFAC * plane + (size_t)iy * 32 * M * NFAC;
	const cx<double>* ls = lsc + (((size_t)g * 2 + c) * Ny + iy) * 2;
	const cx<double> r0 = ls[0], rden = ls[1];
	const int i0 = lane * M;
	const cx<R> one = mk<R>(1, 0), zero = mk<R>(0, 0);
	const Stencil<R> st{coef + (size_t)g * coef_set_size(N), N, Nx, Ny};
	const cx<R>* f0 = src + (size_t)s0 * 2 * N;
	// right-hand sides, coalesced (point e = lane + 32 t), into the lane-chunk layout of buf; the
	// fixed trip count (rolled, unroll 2 and 4 measured slower on GB300) beats a loop to n_unk
#pragma unroll 1
	for(int t = 0; t < M; t++) {
		const int e = lane + 32 * t;
		if(e < n_unk) {
			cx<R> r[KS];
			composite_m<R, KIND, KS>(st, c, e, iy, f0, r);
#pragma unroll
			for(int j = 0; j < KS; j++) buf[j * PITCH + (e / M) * (M + 1) + e % M] = r[j];
		}
	}
	__syncwarp();
	// Local pass over the lane's chunk: the right-hand sides b (written back over the stencil
	// values in buf), the zero-carry forward values d0 and the three maps that finish the line
	// after one combine:
	//   forward   D_out = P * D_in + d0_end                  (P = product of a)
	//   sum       sum_i w_i d_i = S0 + S1 * D_in
	//   backward  x_start = Cp * X_in + G0 + G1 * D_in       (Cp = product of c)
	// P, S1, G1 and Cp do not depend on the slot. The chunk values live in shared memory, not
	// in registers.
	cx<R> d0[KS], S0[KS], G0[KS];
	cx<R> P = one, S1 = zero, G1 = zero, Cp = one;
#pragma unroll
	for(int j = 0; j < KS; j++) { d0[j] = zero; S0[j] = zero; G0[j] = zero; }
	cx<R>* vb = buf + lane * (M + 1);
#pragma unroll
	for(int k = 0; k < M; k++) {
		if(i0 + k < n_unk) {
			const cx<R> a = Fc[(k * NFAC + F_A) * 32 + lane], rb = Fc[(k * NFAC + F_RB) * 32 + lane];
			const cx<R> w = Fc[(k * NFAC + F_W) * 32 + lane], cc = Fc[(k * NFAC + F_C) * 32 + lane];
			P = a * P;
			S1 = cfma(w, P, S1);
			G1 = cfma(Cp, P, G1);
#pragma unroll
			for(int j = 0; j < KS; j++) {
				const cx<R> b = vb[j * PITCH + k] * rb;
				vb[j * PITCH + k] = b;
				d0[j] = cfma(a, d0[j], b);
				S0[j] = cfma(w, d0[j], S0[j]);
				G0[j] = cfma(Cp, d0[j], G0[j]);
			}
			Cp = Cp * cc;
		}
	}
	// One combine across the chunks (lanes): forward carries, Sherman-Morrison factor,
	// backward carries.
	cx<R> din[KS], xin[KS], fr[KS];
	line_combine<R, KS>(P, d0, S0, S1, G0, G1, Cp, r0, rden, lane, din, xin, fr);
	// Finish: forward values from the carry, then the backward sweep with the correction.
#pragma unroll
	for(int k = 0; k < M; k++) {
		if(i0 + k < n_unk) {
			const cx<R> a = Fc[(k * NFAC + F_A) * 32 + lane];
#pragma unroll
			for(int j = 0; j < KS; j++) { din[j] = cfma(a, din[j], vb[j * PITCH + k]); vb[j * PITCH + k] = din[j]; }
		}
	}
#pragma unroll
	for(int k = M - 1; k >= 0; k--) {
		if(i0 + k < n_unk) {
			const cx<R> cc = Fc[(k * NFAC + F_C) * 32 + lane], cr = Fc[(k * NFAC + F_COR) * 32 + lane];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				xin[j] = cfma(cc, xin[j], vb[j * PITCH + k]);
				vb[j * PITCH + k] = cfnma(fr[j], cr, xin[j]);
			}
		}
	}
	// the explicit-step solves never accumulate; the accumulating ones load the accumulator inputs
	// of several points before storing any (their latency would otherwise be paid point by point)
	const bool acc = KIND != ST_EXPL_Y && acc_out;
	if(!TOUT) {
	__syncwarp();
	constexpr int U = 3;
#pragma unroll 1
	for(int t0 = 0; t0 <= M; t0 += U) {
		cx<R> a[U][KS];
		if(acc) {
#pragma unroll
			for(int u = 0; u < U; u++) {
				const int e = lane + 32 * (t0 + u);
				if(t0 + u <= M && e < Nx)
#pragma unroll
					for(int j = 0; j < KS; j++) {
						const size_t o = (size_t)(s0 + j) * 2 * N + (size_t)c * N + (size_t)iy * Nx + e;
						a[u][j] = acc_in2 ? acc_in[o] + acc_in2[o] : acc_in[o];
					}
			}
		}
#pragma unroll
		for(int u = 0; u < U; u++) {
			const int e = lane + 32 * (t0 + u);
			if(t0 + u <= M && e < Nx) {
				const int ee = e == Nx - 1 ? 0 : e;
#pragma unroll
				for(int j = 0; j < KS; j++) {
					const size_t o = (size_t)(s0 + j) * 2 * N + (size_t)c * N + (size_t)iy * Nx + e;
					const cx<R> x = buf[j * PITCH + (ee / M) * (M + 1) + ee % M];
					if(dst) dst[o] = x;
					if(acc) acc_out[o] = a[u][j] + x;
				}
			}
		}
	}
	}
	}  // iy < Ny
	if(TOUT) {
		__syncthreads();
		const cx<R>* bufs = reinterpret_cast<const cx<R>*>(smem_raw);
		const bool acc = KIND != ST_EXPL_Y && acc_out;
		constexpr int U = 4, BT = 32 * LT;
		for(int t0 = threadIdx.x; t0 < Nx * LT; t0 += U * BT) {
			cx<R> a[U][KS];
			if(acc) {
#pragma unroll
				for(int u = 0; u < U; u++) {
					const int t = t0 + u * BT, e = t / LT, line = blockIdx.x * LT + t % LT;
					if(t < Nx * LT && line < Ny)
#pragma unroll
						for(int j = 0; j < KS; j++) {
							const size_t in = (size_t)(s0 + j) * 2 * N + (size_t)c * N + (size_t)line * Nx + e;
							a[u][j] = acc_in2 ? acc_in[in] + acc_in2[in] : acc_in[in];
						}
				}
			}
#pragma unroll
			for(int u = 0; u < U; u++) {
				const int t = t0 + u * BT, e = t / LT, w = t % LT, line = blockIdx.x * LT + w;
				if(t < Nx * LT && line < Ny) {
					const int ee = e == Nx - 1 ? 0 : e;
					const cx<R>* bw = bufs + (size_t)w * KS * PITCH + (ee / M) * (M + 1) + ee % M;
#pragma unroll
					for(int j = 0; j < KS; j++) {
						const size_t out = (size_t)(s0 + j) * 2 * N + (size_t)(1 - c) * N + (size_t)e * Ny + line;
						const cx<R> x = bw[j * PITCH];
						if(dst) dst[out] = x;
						if(acc) acc_out[out] = a[u][j] + x;
					}
				}
			}
		}
	}
}

// y-line solve in the x-line form: one warp per (column, comp, KS slots of one wavelength), lane l
// owning the rows [l*M, l*M+M) of the column, the chunk maps combined by warp shuffles
// (line_combine) as in k_solve_xc, so that no barrier joins the warps of a line. A block of LT
// warps takes LT adjacent columns: its threads form the right-hand sides of every (row, column)
// pair of those columns together (consecutive threads take the columns of a row, so a warp's
// loads are 32-byte row segments of eight rows) into the warps' shared buffers in the lane-chunk
// layout, each warp solves its column, and the block writes the results back row by row. The
// factor planes keep the plain [row][column] layout (each 32-byte sector of a row serves the LT
// warps of the block). KIND: ST_EXPL_X (explicit x half-step) or ST_WOOD_Y (Woodbury term).
// Restates BlockSparseMatrixDY::shifted_block_vmult_inv (BlockSparseMatrix.cpp:386-451) with the
// right-hand sides of ParaxialPrimaryEvolutionOperator::apply (ParaxialPrimaryEvolutionOperator.
// cpp:153-209). Outputs: dst = x (may be null), acc_out = (acc_in [+ acc_in2]) + x (may be null).
template <typename R, int M, int KIND, int KS>
__global__ void __launch_bounds__(128, NBPM_XC_MINB(M * KS)) k_solve_yt(Geom G, int nch, const cx<R>* __restrict__ coef,
		const cx<R>* __restrict__ fac, size_t plane, const cx<double>* __restrict__ lsc,
		const cx<R>* __restrict__ src, cx<R>* __restrict__ dst, const cx<R>* acc_in, cx<R>* acc_out,
		const cx<R>* acc_in2) {
	extern __shared__ unsigned char smem_raw[];
	const int LT = blockDim.x / 32;
	const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int x0 = blockIdx.x * LT;
	const int c = blockIdx.y % 2, bc = blockIdx.y / 2;
	const int g = bc / nch, ch = bc % nch;
	const int s0 = g * G.spg + ch * KS;
	const int n_unk = Ny - 1;
	const int PITCH = 32 * (M + 1);
	cx<R>* const bufs = reinterpret_cast<cx<R>*>(smem_raw);
	const Stencil<R> st{coef + (size_t)g * coef_set_size(N), N, Nx, Ny};
	const cx<R>* f0 = src + (size_t)s0 * 2 * N;
	const cx<R> one = mk<R>(1, 0), zero = mk<R>(0, 0);
	// right-hand sides of every (row, column) pair of the block's columns
	for(int e = threadIdx.x; e < n_unk * LT; e += blockDim.x) {
		const int i = e / LT, w = e % LT, x = x0 + w;
		if(x < Nx) {
			cx<R> r[KS];
			composite_m<R, KIND, KS>(st, c, x, i, f0, r);
			cx<R>* b = bufs + (size_t)w * KS * PITCH + (i / M) * (M + 1) + i % M;
#pragma unroll
			for(int j = 0; j < KS; j++) b[j * PITCH] = r[j];
		}
	}
	__syncthreads();
	const int x = x0 + warp;
	if(x < Nx) {
		cx<R>* buf = bufs + (size_t)warp * KS * PITCH;
		const cx<R>* Fc = fac + ((size_t)g * 2 + c) * NFAC * plane + x;
		const cx<double>* ls = lsc + (((size_t)g * 2 + c) * Nx + x) * 2;
		const cx<double> r0 = ls[0], rden = ls[1];
		const int i0 = lane * M;
		cx<R> d0[KS], S0[KS], G0[KS];
		cx<R> P = one, S1 = zero, G1 = zero, Cp = one;
#pragma unroll
		for(int j = 0; j < KS; j++) { d0[j] = zero; S0[j] = zero; G0[j] = zero; }
		cx<R>* vb = buf + lane * (M + 1);
#pragma unroll
		for(int k = 0; k < M; k++) {
			if(i0 + k < n_unk) {
				const size_t q = (size_t)(i0 + k) * Nx;
				const cx<R> a = Fc[F_A * plane + q], rb = Fc[F_RB * plane + q];
				const cx<R> w = Fc[F_W * plane + q], cc = Fc[F_C * plane + q];
				P = a * P;
				S1 = cfma(w, P, S1);
				G1 = cfma(Cp, P, G1);
#pragma unroll
				for(int j = 0; j < KS; j++) {
					const cx<R> b = vb[j * PITCH + k] * rb;
					vb[j * PITCH + k] = b;
					d0[j] = cfma(a, d0[j], b);
					S0[j] = cfma(w, d0[j], S0[j]);
					G0[j] = cfma(Cp, d0[j], G0[j]);
				}
				Cp = Cp * cc;
			}
		}
		cx<R> din[KS], xin[KS], fr[KS];
		line_combine<R, KS>(P, d0, S0, S1, G0, G1, Cp, r0, rden, lane, din, xin, fr);
#pragma unroll
		for(int k = 0; k < M; k++) {
			if(i0 + k < n_unk) {
				const cx<R> a = Fc[F_A * plane + (size_t)(i0 + k) * Nx];
#pragma unroll
				for(int j = 0; j < KS; j++) { din[j] = cfma(a, din[j], vb[j * PITCH + k]); vb[j * PITCH + k] = din[j]; }
			}
		}
#pragma unroll
		for(int k = M - 1; k >= 0; k--) {
			if(i0 + k < n_unk) {
				const size_t q = (size_t)(i0 + k) * Nx;
				const cx<R> cc = Fc[F_C * plane + q], cr = Fc[F_COR * plane + q];
#pragma unroll
				for(int j = 0; j < KS; j++) {
					xin[j] = cfma(cc, xin[j], vb[j * PITCH + k]);
					vb[j * PITCH + k] = cfnma(fr[j], cr, xin[j]);
				}
			}
		}
	}
	__syncthreads();
	// results, row by row (row Ny-1 repeats row 0)
	for(int e = threadIdx.x; e < Ny * LT; e += blockDim.x) {
		const int i = e / LT, w = e % LT, xo = x0 + w;
		if(xo >= Nx) continue;
		const int ii = i == Ny - 1 ? 0 : i;
		const cx<R>* b = bufs + (size_t)w * KS * PITCH + (ii / M) * (M + 1) + ii % M;
#pragma unroll
		for(int j = 0; j < KS; j++) {
			const size_t off = (size_t)(s0 + j) * 2 * N + (size_t)c * N + (size_t)i * Nx + xo;
			const cx<R> v = b[j * PITCH];
			if(dst) dst[off] = v;
			if(KIND != ST_EXPL_X && acc_out) acc_out[off] = (acc_in2 ? acc_in[off] + acc_in2[off] : acc_in[off]) + v;
		}
	}
}

// Whether k_solve_yc<M, KS, MAXT> keeps its chunk values in shared memory: the values
// (KS*M*MAXT complex) and the combine arrays ((4 + 3 KS)*MAXT + 32 KS complex) within 224 KiB.
__host__ __device__ constexpr bool yc_values_in_smem(int M, int KS, int MAXT, int csize) {
	return ((long)KS * M * MAXT + (4L + 3L * KS) * MAXT + 32L * KS) * csize <= 224L * 1024;
}

// Combine of the y-chunk maps of a block (32 columns x WY chunks; shared arrays at
// [chunk][column], per-slot arrays at [slot][chunk][column]): warp w combines columns
// w, w + WY, ... with its lanes indexing the chunks (line_combine), and leaves per chunk the
// forward and backward entering values in sD0 / sG0 and per column the Sherman-Morrison
// factor in sF.
template <typename R, int KS>
__device__ __forceinline__ void ycol_combine(const cx<R>* sP, const cx<R>* sS1, const cx<R>* sG1, const cx<R>* sCp,
		cx<R>* sD0, const cx<R>* sS0, cx<R>* sG0, cx<R>* sF, int WY, int w, int lane, int ix0, int Nx,
		const cx<double>* ls) {
	const int SZ = WY * 32;
	const cx<R> one = mk<R>(1, 0), zero = mk<R>(0, 0);
	for(int col = w; col < 32; col += WY) {
		if(ix0 + col >= Nx) continue;  // uniform across the warp
		const bool ok = lane < WY;
		const int e = lane * 32 + col;
		const cx<R> P = ok ? sP[e] : one, S1 = ok ? sS1[e] : zero, G1 = ok ? sG1[e] : zero, Cp = ok ? sCp[e] : one;
		cx<R> d0[KS], S0[KS], G0[KS], din[KS], xin[KS], fr[KS];
#pragma unroll
		for(int j = 0; j < KS; j++) {
			d0[j] = ok ? sD0[j * SZ + e] : zero;
			S0[j] = ok ? sS0[j * SZ + e] : zero;
			G0[j] = ok ? sG0[j * SZ + e] : zero;
		}
		const cx<double> r0 = ls[(size_t)(ix0 + col) * 2], rden = ls[(size_t)(ix0 + col) * 2 + 1];
		line_combine<R, KS>(P, d0, S0, S1, G0, G1, Cp, r0, rden, lane, din, xin, fr);
		if(ok) {
#pragma unroll
			for(int j = 0; j < KS; j++) { sD0[j * SZ + e] = din[j]; sG0[j * SZ + e] = xin[j]; }
		}
		if(lane == 0) {
#pragma unroll
			for(int j = 0; j < KS; j++) sF[j * 32 + col] = fr[j];
		}
	}
}

// y-line solve fused with its right-hand side (KIND: explicit x half-step or y Woodbury term),
// chunked parallel form: block = 32 adjacent columns (lanes, coalesced) x WY warps for KS
// slots of one wavelength; warp w owns the rows [w*M, w*M+M) of the 32 lines for all KS
// slots. One pass builds the chunk maps, one combine (ycol_combine) joins them across the
// warps, one pass finishes the lines. MAXT: block size the instance is compiled for (512, or
// 1024 for 32 warps of short chunks).
template <typename R, int M, int KIND, int KS, int MAXT = 512>
__global__ void __launch_bounds__(MAXT, NBPM_YC_MINB) k_solve_yc(Geom G, int slot0, int nch, const cx<R>* __restrict__ coef,
		const cx<R>* __restrict__ fac, size_t plane, const cx<double>* __restrict__ lsc,
		const cx<R>* __restrict__ src, cx<R>* __restrict__ dst, const cx<R>* acc_in, cx<R>* acc_out,
		const cx<R>* acc_in2) {
	extern __shared__ unsigned char smem_raw[];
	const int WY = blockDim.y;
	const int lane = threadIdx.x, w = threadIdx.y;
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int ix = blockIdx.x * 32 + lane;
	const bool col = ix < Nx;
	const int c = blockIdx.y % 2, bc = blockIdx.y / 2;
	const int g = bc / nch, ch = bc % nch;
	const int s0 = g * G.spg + ch * KS;
	const int n_unk = Ny - 1;
	const int SZ = WY * 32;
	cx<R>* sP = reinterpret_cast<cx<R>*>(smem_raw);  // [WY][32] each
	cx<R>* sS1 = sP + SZ;
	cx<R>* sG1 = sS1 + SZ;
	cx<R>* sCp = sG1 + SZ;
	cx<R>* sD0 = sCp + SZ;                            // [KS][WY][32] each
	cx<R>* sS0 = sD0 + KS * SZ;
	cx<R>* sG0 = sS0 + KS * SZ;
	cx<R>* sF = sG0 + KS * SZ;                        // [KS][32]
	// chunk values in shared memory ([KS][M][WY][32]) when they fit beside the combine arrays,
	// else in registers
	constexpr bool VS = yc_values_in_smem(M, KS, MAXT, (int)sizeof(cx<R>));
	cx<R>* sV = sF + KS * 32;
	const cx<R>* Fc = fac + ((size_t)g * 2 + c) * NFAC * plane;
	const int i0 = w * M;
	const cx<R> one = mk<R>(1, 0), zero = mk<R>(0, 0);
	const Stencil<R> st{coef + (size_t)g * coef_set_size(N), N, Nx, Ny};
	const cx<R>* f0 = src + (size_t)s0 * 2 * N;
	// chunk pass: right-hand sides b (kept in v) and the chunk maps of line_combine
	cx<R> v[VS ? 1 : KS][VS ? 1 : M];
	auto V = [&](int j, int k) -> cx<R>& { return VS ? sV[((j * M + k) * WY + w) * 32 + lane] : v[VS ? 0 : j][VS ? 0 : k]; };
	cx<R> d0[KS], S0[KS], G0[KS];
	cx<R> P = one, S1 = zero, G1 = zero, Cp = one;
#pragma unroll
	for(int j = 0; j < KS; j++) { d0[j] = zero; S0[j] = zero; G0[j] = zero; }
	// chunk values in shared memory need no compile-time row index: unroll by 2 in the 16-warp
	// blocks (measured faster on GB300), fully in the 32-warp ones
	constexpr int U1 = (VS && MAXT <= 512 && M >= 2) ? 2 : M;
#pragma unroll U1
	for(int k = 0; k < M; k++) {
		const int i = i0 + k;
#pragma unroll
		for(int j = 0; j < KS; j++) V(j, k) = zero;
		if(col && i < n_unk) {
			const size_t q = (size_t)ix + (size_t)Nx * i;
			const cx<R> a = Fc[F_A * plane + q], rb = Fc[F_RB * plane + q];
			const cx<R> wv = Fc[F_W * plane + q], cc = Fc[F_C * plane + q];
			cx<R> r[KS];
			composite_m<R, KIND, KS>(st, c, ix, i, f0, r);
			P = a * P;
			S1 = cfma(wv, P, S1);
			G1 = cfma(Cp, P, G1);
#pragma unroll
			for(int j = 0; j < KS; j++) {
				const cx<R> b = r[j] * rb;
				V(j, k) = b;
				d0[j] = cfma(a, d0[j], b);
				S0[j] = cfma(wv, d0[j], S0[j]);
				G0[j] = cfma(Cp, d0[j], G0[j]);
			}
			Cp = Cp * cc;
		}
	}
	{
		const int e = w * 32 + lane;
		sP[e] = P; sS1[e] = S1; sG1[e] = G1; sCp[e] = Cp;
#pragma unroll
		for(int j = 0; j < KS; j++) { sD0[j * SZ + e] = d0[j]; sS0[j * SZ + e] = S0[j]; sG0[j * SZ + e] = G0[j]; }
	}
	__syncthreads();
	ycol_combine<R, KS>(sP, sS1, sG1, sCp, sD0, sS0, sG0, sF, WY, w, lane, blockIdx.x * 32, Nx,
		lsc + ((size_t)g * 2 + c) * Nx * 2);
	__syncthreads();
	if(!col) return;
	cx<R> d[KS], x[KS], fr[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) {
		d[j] = sD0[j * SZ + w * 32 + lane];
		x[j] = sG0[j * SZ + w * 32 + lane];
		fr[j] = sF[j * 32 + lane];
	}
#pragma unroll
	for(int k = 0; k < M; k++) {
		const int i = i0 + k;
		if(i < n_unk) {
			const cx<R> a = Fc[F_A * plane + (size_t)ix + (size_t)Nx * i];
#pragma unroll
			for(int j = 0; j < KS; j++) { d[j] = cfma(a, d[j], V(j, k)); V(j, k) = d[j]; }
		}
	}
#pragma unroll
	for(int k = M - 1; k >= 0; k--) {
		const int i = i0 + k;
		if(i < n_unk) {
			const size_t q = (size_t)ix + (size_t)Nx * i;
			const cx<R> cc = Fc[F_C * plane + q], cr = Fc[F_COR * plane + q];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				x[j] = cfma(cc, x[j], V(j, k));
				const cx<R> y = cfnma(fr[j], cr, x[j]);
				const size_t off = (size_t)(s0 + j) * 2 * N + (size_t)c * N;
				if(dst) dst[off + q] = y;
				// the explicit-step solves never accumulate
				if(KIND != ST_EXPL_X && acc_out)
					acc_out[off + q] = (acc_in2 ? acc_in[off + q] + acc_in2[off + q] : acc_in[off + q]) + y;
				if(i == 0) {
					const size_t qe = (size_t)ix + (size_t)Nx * (Ny - 1);
					if(dst) dst[off + qe] = y;
					if(KIND != ST_EXPL_X && acc_out)
						acc_out[off + qe] = (acc_in2 ? acc_in[off + qe] + acc_in2[off + qe] : acc_in[off + qe]) + y;
				}
			}
		}
	}
}

// y-line solve fused with its right-hand side, sequential form: one thread per (column, KS
// slots of one wavelength), both field components. Consecutive threads take consecutive columns,
// so every load and store of a row is coalesced. The forward sweep
//   d_i = alpha_i d_{i-1} + b_i / beta_i,   S = sum_i w_i d_i
// stores d_i in scr (a field-sized buffer that none of the inputs alias: the output buffer
// itself when there is one), the Sherman-Morrison factor f = (S - r0 d_{n-1}) rden is formed in
// FP64, and the backward sweep x_i = d_i - gamma_i x_{i+1} turns d into the solution
// x_i - f corr_i in place. Every thread is independent: no barriers, no cross-chunk combine,
// and a tenth of the instructions per point of the chunked form (the stencil taps of the
// neighbouring columns come from L1). Restates BlockSparseMatrixDY::shifted_block_vmult_inv
// (BlockSparseMatrix.cpp:386-451) with the right-hand side of ParaxialPrimaryEvolutionOperator::
// apply (ParaxialPrimaryEvolutionOperator.cpp:153-209) for KIND = ST_EXPL_X (explicit x
// half-step) or ST_WOOD_Y (Woodbury term). Outputs: dst = x (may be null), acc_out =
// (acc_in [+ acc_in2]) + x (may be null); row Ny-1 receives row 0 (period Ny-1).
template <typename R, int KIND, int KS>
__global__ void __launch_bounds__(128) k_solve_yq(Geom G, int nch, const cx<R>* __restrict__ coef,
		const cx<R>* __restrict__ fac, size_t plane, const cx<double>* __restrict__ lsc,
		const cx<R>* __restrict__ src, cx<R>* scr, cx<R>* dst, const cx<R>* acc_in, cx<R>* acc_out,
		const cx<R>* acc_in2) {
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int ix = blockIdx.x * blockDim.x + threadIdx.x;
	if(ix >= Nx) return;
	const int g = blockIdx.y / nch, ch = blockIdx.y % nch;
	const int s0 = g * G.spg + ch * KS;
	const int n = Ny - 1;
	const size_t ss = 2 * (size_t)N;
	const Stencil<R> st{coef + (size_t)g * coef_set_size(N), N, Nx, Ny};
	const cx<R>* f0 = src + (size_t)s0 * ss;
	const cx<R>* F0 = fac + ((size_t)g * 2 + 0) * NFAC * plane;
	const cx<R>* F1 = fac + ((size_t)g * 2 + 1) * NFAC * plane;
	cx<R>* sc = scr + (size_t)s0 * ss;
	const cx<R> zero = mk<R>(0, 0);
	cx<R> d0[KS], d1[KS], a0[KS], a1[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) { d0[j] = zero; d1[j] = zero; a0[j] = zero; a1[j] = zero; }
#pragma unroll 2
	for(int i = 0; i < n; i++) {
		const size_t q = (size_t)ix + (size_t)Nx * i;
		cx<R> r0[KS], r1[KS];
		composite_m<R, KIND, KS>(st, 0, ix, i, f0, r0);
		composite_m<R, KIND, KS>(st, 1, ix, i, f0, r1);
		const cx<R> A0 = F0[F_A * plane + q], B0 = F0[F_RB * plane + q], W0 = F0[F_W * plane + q];
		const cx<R> A1 = F1[F_A * plane + q], B1 = F1[F_RB * plane + q], W1 = F1[F_W * plane + q];
#pragma unroll
		for(int j = 0; j < KS; j++) {
			const cx<R> b0 = r0[j] * B0, b1 = r1[j] * B1;
			d0[j] = cfma(A0, d0[j], b0);
			d1[j] = cfma(A1, d1[j], b1);
			a0[j] = cfma(W0, d0[j], a0[j]);
			a1[j] = cfma(W1, d1[j], a1[j]);
			sc[j * ss + q] = d0[j];
			sc[j * ss + N + q] = d1[j];
		}
	}
	const cx<double>* l0 = lsc + (((size_t)g * 2 + 0) * Nx + ix) * 2;
	const cx<double>* l1 = lsc + (((size_t)g * 2 + 1) * Nx + ix) * 2;
	const cx<double> r00 = l0[0], rd0 = l0[1], r01 = l1[0], rd1 = l1[1];
	cx<R> fr0[KS], fr1[KS], x0[KS], x1[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) {
		fr0[j] = cvt<R>((cvt<double>(a0[j]) - r00 * cvt<double>(d0[j])) * rd0);
		fr1[j] = cvt<R>((cvt<double>(a1[j]) - r01 * cvt<double>(d1[j])) * rd1);
		x0[j] = zero;
		x1[j] = zero;
	}
	const size_t qe = (size_t)ix + (size_t)Nx * n;
#pragma unroll 2
	for(int i = n - 1; i >= 0; i--) {
		const size_t q = (size_t)ix + (size_t)Nx * i;
		const cx<R> C0 = F0[F_C * plane + q], K0 = F0[F_COR * plane + q];
		const cx<R> C1 = F1[F_C * plane + q], K1 = F1[F_COR * plane + q];
#pragma unroll
		for(int j = 0; j < KS; j++) {
			const size_t o0 = (size_t)(s0 + j) * ss + q, o1 = o0 + N;
			x0[j] = cfma(C0, x0[j], sc[j * ss + q]);
			x1[j] = cfma(C1, x1[j], sc[j * ss + N + q]);
			const cx<R> y0 = x0[j] - fr0[j] * K0, y1 = x1[j] - fr1[j] * K1;
			if(dst) { dst[o0] = y0; dst[o1] = y1; }
			if(KIND != ST_EXPL_X && acc_out) {
				acc_out[o0] = (acc_in2 ? acc_in[o0] + acc_in2[o0] : acc_in[o0]) + y0;
				acc_out[o1] = (acc_in2 ? acc_in[o1] + acc_in2[o1] : acc_in[o1]) + y1;
			}
			if(i == 0) {
				const size_t e0 = (size_t)(s0 + j) * ss + qe, e1 = e0 + N;
				if(dst) { dst[e0] = y0; dst[e1] = y1; }
				if(KIND != ST_EXPL_X && acc_out) {
					acc_out[e0] = (acc_in2 ? acc_in[e0] + acc_in2[e0] : acc_in[e0]) + y0;
					acc_out[e1] = (acc_in2 ? acc_in[e1] + acc_in2[e1] : acc_in[e1]) + y1;
				}
			}
		}
	}
}

// x-line solve for long lines: one block of W warps per line, 32*W chunks of M points (the
// chunk-interleaved factor layout with 32*W chunks). Within a warp the chunk maps combine with
// shuffles as in k_solve_xc, across the warps of the line through shared memory.
// acc_in2 (may be null): a second accumulator input, acc_out = (acc_in + acc_in2) + x. TOUT: the
// results go out transposed with the components exchanged ((c, iy, e) -> (1 - c, e, iy) of an
// Ny x Nx plane), as in k_solve_xc.
template <typename R, int M, int KIND, int KS, bool TOUT = false>
__global__ void __launch_bounds__(256) k_solve_xw(Geom G, int slot0, int nch, const cx<R>* __restrict__ coef,
		const cx<R>* __restrict__ fac, size_t plane, const cx<double>* __restrict__ lsc,
		const cx<R>* __restrict__ src, cx<R>* __restrict__ dst, const cx<R>* acc_in, cx<R>* acc_out,
		const cx<R>* acc_in2) {
	extern __shared__ unsigned char smem_raw[];
	const int W = blockDim.x / 32;
	const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int iy = blockIdx.x;
	const int c = blockIdx.y % 2, bc = blockIdx.y / 2;
	const int g = bc / nch, ch = bc % nch;
	const int s0 = g * G.spg + ch * KS;
	const int n_unk = Nx - 1;
	const int CH = 32 * W;
	const int ci = warp * 32 + lane;
	const int PITCH = CH * (M + 1);
	cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw);  // [KS][CH][M+1]
	cx<R>* sA = buf + KS * PITCH;                     // [KS][W]
	cx<R>* sB = sA + KS * W;
	cx<R>* sD = sB + KS * W;
	cx<R>* sP = sD + KS * W;
	cx<R>* sX = sP + KS * W;                          // [KS][2]: d at the last unknown, fr
	const cx<R>* Fc = fac + ((size_t)g * 2 + c) * NFAC * plane + (size_t)iy * CH * M * NFAC;
	const cx<double>* ls = lsc + (((size_t)g * 2 + c) * Ny + iy) * 2;
	const cx<double> r0 = ls[0], rden = ls[1];
	const int i0 = ci * M;
	const int last = n_unk - 1;
	const cx<R> one = mk<R>(1, 0), zero = mk<R>(0, 0);
	const Stencil<R> st{coef + (size_t)g * coef_set_size(N), N, Nx, Ny};
	const cx<R>* f0 = src + (size_t)s0 * 2 * N;
	for(int e = threadIdx.x; e < n_unk; e += blockDim.x) {
		cx<R> r[KS];
		composite_m<R, KIND, KS>(st, c, e, iy, f0, r);
#pragma unroll
		for(int j = 0; j < KS; j++) buf[j * PITCH + (e / M) * (M + 1) + e % M] = r[j];
	}
	__syncthreads();
	cx<R> v[KS][M];
	cx<R> A[KS], B[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) { A[j] = one; B[j] = zero; }
#pragma unroll
	for(int k = 0; k < M; k++) {
		bool ok = i0 + k < n_unk;
		cx<R> a = zero, rb = zero;
		if(ok) { a = Fc[(k * NFAC + F_A) * CH + ci]; rb = Fc[(k * NFAC + F_RB) * CH + ci]; }
#pragma unroll
		for(int j = 0; j < KS; j++) {
			v[j][k] = zero;
			if(ok) {
				cx<R> b = buf[j * PITCH + ci * (M + 1) + k] * rb;
				v[j][k] = b;
				B[j] = cfma(a, B[j], b);
				A[j] = a * A[j];
			}
		}
	}
	// forward: inclusive scan within the warp, then the warps' totals in order
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
#pragma unroll
		for(int j = 0; j < KS; j++) {
			cx<R> Ap = shfl_up_c(A[j], o), Bp = shfl_up_c(B[j], o);
			if(lane >= o) { B[j] = A[j] * Bp + B[j]; A[j] = A[j] * Ap; }
		}
	}
	if(lane == 31) {
#pragma unroll
		for(int j = 0; j < KS; j++) { sA[j * W + warp] = A[j]; sB[j * W + warp] = B[j]; }
	}
	__syncthreads();
	if(threadIdx.x < KS) {
		int j = threadIdx.x;
		cx<R> D = zero;
		for(int ww = 0; ww < W; ww++) {
			sD[j * W + ww] = D;
			D = sA[j * W + ww] * D + sB[j * W + ww];
		}
	}
	__syncthreads();
	cx<R> d[KS], acc[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) {
		cx<R> Ae = shfl_up_c(A[j], 1), Be = shfl_up_c(B[j], 1);
		if(lane == 0) { Ae = one; Be = zero; }
		d[j] = Ae * sD[j * W + warp] + Be;
		acc[j] = zero;
	}
#pragma unroll
	for(int k = 0; k < M; k++) {
		if(i0 + k < n_unk) {
			cx<R> a = Fc[(k * NFAC + F_A) * CH + ci], w = Fc[(k * NFAC + F_W) * CH + ci];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				d[j] = cfma(a, d[j], v[j][k]);
				v[j][k] = d[j];
				acc[j] = cfma(w, d[j], acc[j]);
			}
			if(i0 + k == last) {
#pragma unroll
				for(int j = 0; j < KS; j++) sX[2 * j] = d[j];
			}
		}
	}
#pragma unroll
	for(int j = 0; j < KS; j++) {
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) acc[j] += shfl_xor_c(acc[j], o);
		if(lane == 0) sP[j * W + warp] = acc[j];
	}
	__syncthreads();
	if(threadIdx.x < KS) {
		int j = threadIdx.x;
		cx<R> tot = zero;
		for(int ww = 0; ww < W; ww++) tot += sP[j * W + ww];
		sX[2 * j + 1] = cvt<R>((cvt<double>(tot) - r0 * cvt<double>(sX[2 * j])) * rden);
	}
	// backward: chunk maps, inclusive scan from the line's end
#pragma unroll
	for(int j = 0; j < KS; j++) { A[j] = one; B[j] = zero; }
#pragma unroll
	for(int k = M - 1; k >= 0; k--) {
		if(i0 + k < n_unk) {
			cx<R> cc = Fc[(k * NFAC + F_C) * CH + ci];
#pragma unroll
			for(int j = 0; j < KS; j++) { B[j] = cfma(cc, B[j], v[j][k]); A[j] = cc * A[j]; }
		}
	}
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
#pragma unroll
		for(int j = 0; j < KS; j++) {
			cx<R> An = shfl_down_c(A[j], o), Bn = shfl_down_c(B[j], o);
			if(lane + o < 32) { B[j] = A[j] * Bn + B[j]; A[j] = A[j] * An; }
		}
	}
	__syncthreads();  // sD of the forward pass has been read
	if(lane == 0) {
#pragma unroll
		for(int j = 0; j < KS; j++) { sA[j * W + warp] = A[j]; sB[j * W + warp] = B[j]; }
	}
	__syncthreads();
	if(threadIdx.x < KS) {
		int j = threadIdx.x;
		cx<R> D = zero;
		for(int ww = W - 1; ww >= 0; ww--) {
			sD[j * W + ww] = D;
			D = sA[j * W + ww] * D + sB[j * W + ww];
		}
	}
	__syncthreads();
	cx<R> fr[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) {
		fr[j] = sX[2 * j + 1];
		cx<R> An = shfl_down_c(A[j], 1), Bn = shfl_down_c(B[j], 1);
		if(lane == 31) { An = one; Bn = zero; }
		d[j] = An * sD[j * W + warp] + Bn;
	}
#pragma unroll
	for(int k = M - 1; k >= 0; k--) {
		if(i0 + k < n_unk) {
			cx<R> cc = Fc[(k * NFAC + F_C) * CH + ci], cr = Fc[(k * NFAC + F_COR) * CH + ci];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				d[j] = cfma(cc, d[j], v[j][k]);
				buf[j * PITCH + ci * (M + 1) + k] = cfnma(fr[j], cr, d[j]);
			}
		}
	}
	__syncthreads();
	// write-out: the accumulator inputs of several points are loaded before any store
	constexpr int U = 4;
	for(int e0 = threadIdx.x; e0 < Nx; e0 += U * blockDim.x) {
		cx<R> a[U][KS];
		if(acc_out) {
#pragma unroll
			for(int u = 0; u < U; u++) {
				const int e = e0 + u * blockDim.x;
				if(e < Nx)
#pragma unroll
					for(int j = 0; j < KS; j++) {
						const size_t o = (size_t)(s0 + j) * 2 * N + (size_t)c * N + (size_t)iy * Nx + e;
						a[u][j] = acc_in2 ? acc_in[o] + acc_in2[o] : acc_in[o];
					}
			}
		}
#pragma unroll
		for(int u = 0; u < U; u++) {
			const int e = e0 + u * blockDim.x;
			if(e < Nx) {
				const int ee = e == Nx - 1 ? 0 : e;
#pragma unroll
				for(int j = 0; j < KS; j++) {
					const cx<R> x = buf[j * PITCH + (ee / M) * (M + 1) + ee % M];
					const size_t o = TOUT ? (size_t)(s0 + j) * 2 * N + (size_t)(1 - c) * N + iy + (size_t)e * Ny
						: (size_t)(s0 + j) * 2 * N + (size_t)c * N + (size_t)iy * Nx + e;
					if(dst) dst[o] = x;
					if(acc_out) acc_out[o] = a[u][j] + x;
				}
			}
		}
	}
}

// x-line solve with the chunk values in the warp's shared-memory buffer instead of registers
// (same algorithm and layout as k_solve_xc): for long lines (large M) the per-thread state
// stays small, so more warps stay resident.
template <typename R, int KIND, int KS>
__global__ void __launch_bounds__(128) k_solve_xs(Geom G, int slot0, int nch, int M, const cx<R>* __restrict__ coef,
		const cx<R>* __restrict__ fac, size_t plane, const cx<double>* __restrict__ lsc,
		const cx<R>* __restrict__ src, cx<R>* __restrict__ dst, const cx<R>* acc_in, cx<R>* acc_out) {
	extern __shared__ unsigned char smem_raw[];
	const int LT = blockDim.x / 32;
	const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int iy = blockIdx.x * LT + warp;
	if(iy >= Ny) return;
	const int c = blockIdx.y % 2, bc = blockIdx.y / 2;
	const int g = bc / nch, ch = bc % nch;
	const int s0 = g * G.spg + ch * KS;
	const int n_unk = Nx - 1;
	const int PITCH = 32 * (M + 1);
	cx<R>* buf = reinterpret_cast<cx<R>*>(smem_raw) + (size_t)warp * KS * PITCH;
	const cx<R>* Fc = fac + ((size_t)g * 2 + c) * NFAC * plane + (size_t)iy * 32 * M * NFAC;
	const cx<double>* ls = lsc + (((size_t)g * 2 + c) * Ny + iy) * 2;
	const cx<double> r0 = ls[0], rden = ls[1];
	const int i0 = lane * M;
	const int last = n_unk - 1, lane_last = last / M, k_last = last % M;
	const cx<R> one = mk<R>(1, 0), zero = mk<R>(0, 0);
	const Stencil<R> st{coef + (size_t)g * coef_set_size(N), N, Nx, Ny};
	const cx<R>* f0 = src + (size_t)s0 * 2 * N;
	for(int e = lane; e < n_unk; e += 32) {
		cx<R> r[KS];
		composite_m<R, KIND, KS>(st, c, e, iy, f0, r);
#pragma unroll
		for(int j = 0; j < KS; j++) buf[j * PITCH + (e / M) * (M + 1) + e % M] = r[j];
	}
	__syncwarp();
	auto V = [&](int j, int k) -> cx<R>& { return buf[j * PITCH + lane * (M + 1) + k]; };
	cx<R> A[KS], B[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) { A[j] = one; B[j] = zero; }
	for(int k = 0; k < M; k++) {
		if(i0 + k < n_unk) {
			cx<R> a = Fc[(k * NFAC + F_A) * 32 + lane], rb = Fc[(k * NFAC + F_RB) * 32 + lane];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				cx<R> b = V(j, k) * rb;
				V(j, k) = b;
				B[j] = cfma(a, B[j], b);
				A[j] = a * A[j];
			}
		}
	}
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
#pragma unroll
		for(int j = 0; j < KS; j++) {
			cx<R> Ap = shfl_up_c(A[j], o), Bp = shfl_up_c(B[j], o);
			if(lane >= o) { B[j] = A[j] * Bp + B[j]; A[j] = A[j] * Ap; }
		}
	}
	cx<R> d[KS], acc[KS], dl[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) {
		d[j] = shfl_up_c(B[j], 1);
		if(lane == 0) d[j] = zero;
		acc[j] = zero;
		dl[j] = zero;
	}
	for(int k = 0; k < M; k++) {
		if(i0 + k < n_unk) {
			cx<R> a = Fc[(k * NFAC + F_A) * 32 + lane], w = Fc[(k * NFAC + F_W) * 32 + lane];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				d[j] = cfma(a, d[j], V(j, k));
				V(j, k) = d[j];
				acc[j] = cfma(w, d[j], acc[j]);
			}
		}
		if(k == k_last) {
#pragma unroll
			for(int j = 0; j < KS; j++) dl[j] = d[j];
		}
	}
	cx<R> fr[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) {
#pragma unroll
		for(int o = 16; o > 0; o >>= 1) acc[j] += shfl_xor_c(acc[j], o);
		dl[j] = shfl_idx_c(dl[j], lane_last);
		fr[j] = cvt<R>((cvt<double>(acc[j]) - r0 * cvt<double>(dl[j])) * rden);
		A[j] = one;
		B[j] = zero;
	}
	for(int k = M - 1; k >= 0; k--) {
		if(i0 + k < n_unk) {
			cx<R> cc = Fc[(k * NFAC + F_C) * 32 + lane];
#pragma unroll
			for(int j = 0; j < KS; j++) { B[j] = cfma(cc, B[j], V(j, k)); A[j] = cc * A[j]; }
		}
	}
#pragma unroll
	for(int o = 1; o < 32; o <<= 1) {
#pragma unroll
		for(int j = 0; j < KS; j++) {
			cx<R> An = shfl_down_c(A[j], o), Bn = shfl_down_c(B[j], o);
			if(lane + o < 32) { B[j] = A[j] * Bn + B[j]; A[j] = A[j] * An; }
		}
	}
#pragma unroll
	for(int j = 0; j < KS; j++) {
		d[j] = shfl_down_c(B[j], 1);
		if(lane == 31) d[j] = zero;
	}
	for(int k = M - 1; k >= 0; k--) {
		if(i0 + k < n_unk) {
			cx<R> cc = Fc[(k * NFAC + F_C) * 32 + lane], cr = Fc[(k * NFAC + F_COR) * 32 + lane];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				d[j] = cfma(cc, d[j], V(j, k));
				V(j, k) = cfnma(fr[j], cr, d[j]);
			}
		}
	}
	__syncwarp();
	for(int j = 0; j < KS; j++) {
		const size_t off = (size_t)(s0 + j) * 2 * N + (size_t)c * N + (size_t)iy * Nx;
		for(int e = lane; e < Nx; e += 32) {
			int ee = e == Nx - 1 ? 0 : e;
			cx<R> x = buf[j * PITCH + (ee / M) * (M + 1) + ee % M];
			if(dst) dst[off + e] = x;
			if(acc_out) acc_out[off + e] = acc_in[off + e] + x;
		}
	}
}

// y-line solve for any Ny (same algorithm as k_solve_yc): block = 32 columns x W warps,
// warp w owns rows [w*M, w*M+M) with M = ceil((Ny-1)/W); the chunk values are kept in the
// scratch array vbuf (field layout, L2-resident while the block runs) instead of registers,
// so neither Ny nor the chunk length is bounded by the register file.
template <typename R, int KIND, int KS>
__global__ void __launch_bounds__(256) k_solve_ys(Geom G, int slot0, int nch, const cx<R>* __restrict__ coef,
		const cx<R>* __restrict__ fac, size_t plane, const cx<double>* __restrict__ lsc,
		const cx<R>* __restrict__ src, cx<R>* __restrict__ dst, const cx<R>* acc_in, cx<R>* acc_out,
		cx<R>* __restrict__ vbuf) {
	extern __shared__ unsigned char smem_raw[];
	const int WY = blockDim.y;
	const int lane = threadIdx.x, w = threadIdx.y;
	const int Nx = G.Nx, Ny = G.Ny, N = G.N;
	const int ix = blockIdx.x * 32 + lane;
	const bool col = ix < Nx;
	const int c = blockIdx.y % 2, bc = blockIdx.y / 2;
	const int g = bc / nch, ch = bc % nch;
	const int s0 = g * G.spg + ch * KS;
	const int n_unk = Ny - 1;
	const int M = (n_unk + WY - 1) / WY;
	const int i0 = w * M, i1 = min(i0 + M, n_unk);
	const int SZ = WY * 32;
	cx<R>* sA = reinterpret_cast<cx<R>*>(smem_raw);  // [KS][WY][32]
	cx<R>* sB = sA + KS * SZ;
	cx<R>* sD = sB + KS * SZ;
	cx<R>* sP = sD + KS * SZ;
	cx<R>* sL = sP + KS * SZ;                         // [KS][32]
	cx<R>* sF = sL + KS * 32;                         // [KS][32]
	const cx<R>* Fc = fac + ((size_t)g * 2 + c) * NFAC * plane;
	const cx<R> one = mk<R>(1, 0), zero = mk<R>(0, 0);
	cx<double> r0 = mk(0.0, 0.0), rden = mk(0.0, 0.0);
	if(col) {
		const cx<double>* ls = lsc + (((size_t)g * 2 + c) * Nx + ix) * 2;
		r0 = ls[0];
		rden = ls[1];
	}
	const Stencil<R> st{coef + (size_t)g * coef_set_size(N), N, Nx, Ny};
	const cx<R>* f0 = src + (size_t)s0 * 2 * N;
	auto va = [&](int j, int i) { return (size_t)(s0 + j) * 2 * N + (size_t)c * N + (size_t)ix + (size_t)Nx * i; };
	cx<R> A[KS], B[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) { A[j] = one; B[j] = zero; }
	if(col) {
		for(int i = i0; i < i1; i++) {
			size_t q = (size_t)ix + (size_t)Nx * i;
			cx<R> a = Fc[F_A * plane + q], rb = Fc[F_RB * plane + q];
			cx<R> r[KS];
			composite_m<R, KIND, KS>(st, c, ix, i, f0, r);
#pragma unroll
			for(int j = 0; j < KS; j++) {
				cx<R> b = r[j] * rb;
				vbuf[va(j, i)] = b;
				B[j] = cfma(a, B[j], b);
				A[j] = a * A[j];
			}
		}
	}
#pragma unroll
	for(int j = 0; j < KS; j++) { sA[j * SZ + w * 32 + lane] = A[j]; sB[j * SZ + w * 32 + lane] = B[j]; }
	__syncthreads();
	if(w == 0) {
		for(int j = 0; j < KS; j++) {
			cx<R> D = zero;
			for(int ww = 0; ww < WY; ww++) {
				sD[j * SZ + ww * 32 + lane] = D;
				D = sA[j * SZ + ww * 32 + lane] * D + sB[j * SZ + ww * 32 + lane];
			}
		}
	}
	__syncthreads();
	cx<R> d[KS], acc[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) { d[j] = sD[j * SZ + w * 32 + lane]; acc[j] = zero; }
	if(col) {
		for(int i = i0; i < i1; i++) {
			size_t q = (size_t)ix + (size_t)Nx * i;
			cx<R> a = Fc[F_A * plane + q], wv = Fc[F_W * plane + q];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				d[j] = cfma(a, d[j], vbuf[va(j, i)]);
				vbuf[va(j, i)] = d[j];
				acc[j] = cfma(wv, d[j], acc[j]);
				if(i == n_unk - 1) sL[j * 32 + lane] = d[j];
			}
		}
	}
#pragma unroll
	for(int j = 0; j < KS; j++) sP[j * SZ + w * 32 + lane] = acc[j];
	__syncthreads();
	if(w == 0) {
		for(int j = 0; j < KS; j++) {
			cx<R> tot = zero;
			for(int ww = 0; ww < WY; ww++) tot += sP[j * SZ + ww * 32 + lane];
			sF[j * 32 + lane] = cvt<R>((cvt<double>(tot) - r0 * cvt<double>(sL[j * 32 + lane])) * rden);
		}
	}
#pragma unroll
	for(int j = 0; j < KS; j++) { A[j] = one; B[j] = zero; }
	if(col) {
		for(int i = i1 - 1; i >= i0; i--) {
			cx<R> cc = Fc[F_C * plane + (size_t)ix + (size_t)Nx * i];
#pragma unroll
			for(int j = 0; j < KS; j++) { B[j] = cfma(cc, B[j], vbuf[va(j, i)]); A[j] = cc * A[j]; }
		}
	}
#pragma unroll
	for(int j = 0; j < KS; j++) { sA[j * SZ + w * 32 + lane] = A[j]; sB[j * SZ + w * 32 + lane] = B[j]; }
	__syncthreads();
	if(w == 0) {
		for(int j = 0; j < KS; j++) {
			cx<R> D = zero;
			for(int ww = WY - 1; ww >= 0; ww--) {
				sD[j * SZ + ww * 32 + lane] = D;
				D = sA[j * SZ + ww * 32 + lane] * D + sB[j * SZ + ww * 32 + lane];
			}
		}
	}
	__syncthreads();
	cx<R> fr[KS];
#pragma unroll
	for(int j = 0; j < KS; j++) { fr[j] = sF[j * 32 + lane]; d[j] = sD[j * SZ + w * 32 + lane]; }
	if(col) {
		for(int i = i1 - 1; i >= i0; i--) {
			size_t q = (size_t)ix + (size_t)Nx * i;
			cx<R> cc = Fc[F_C * plane + q], cr = Fc[F_COR * plane + q];
#pragma unroll
			for(int j = 0; j < KS; j++) {
				d[j] = cfma(cc, d[j], vbuf[va(j, i)]);
				cx<R> x = cfnma(fr[j], cr, d[j]);
				size_t off = (size_t)(s0 + j) * 2 * N + (size_t)c * N;
				if(dst) dst[off + q] = x;
				if(acc_out) acc_out[off + q] = acc_in[off + q] + x;
				if(i == 0) {
					size_t qe = (size_t)ix + (size_t)Nx * (Ny - 1);
					if(dst) dst[off + qe] = x;
					if(acc_out) acc_out[off + qe] = acc_in[off + qe] + x;
				}
			}
		}
	}
}

// Point-wise symmetric 2x2 phase operator (PhaseEvolutionOperator.cpp:14-32).
template <typename R>
__global__ void k_phase(Geom G, int slot0, const cx<R>* __restrict__ coef, cx<R>* F) {
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= G.N) return;
	int s = blockIdx.y;
	int N = G.N;
	int g = (slot0 + s) / G.spg - slot0 / G.spg;
	const cx<R>* C = coef + (size_t)g * coef_set_size(N);
	cx<R> oxx = C[cidx(C_PH + 0, p)], oyy = C[cidx(C_PH + 1, p)], oxy = C[cidx(C_PH + 2, p)];
	cx<R>* f = F + (size_t)s * 2 * N + p;
	cx<R> a = f[0], b = f[N];
	f[0] = oxx * a + oxy * b;
	f[N] = oxy * a + oyy * b;
}

// Transverse translation for tilted incidence (SimpleShiftOperator.cpp:52-93): 4-tap cubic
// interpolation with period Nx-1 / Ny-1 (wrap rule SimpleShiftOperator.h:24-39).
__device__ __forceinline__ int ref_wrap(int i, int n) {
	if(i > n - 2) return i % (n - 1);
	if(i < 0) return i + (1 - i / (n - 1)) * (n - 1);
	return i;
}

template <typename R>
__device__ __forceinline__ void phase_apply(const cx<R>* C, size_t N, int p, cx<R>& a, cx<R>& b) {
	cx<R> oxx = C[cidx(C_PH + 0, p)], oyy = C[cidx(C_PH + 1, p)], oxy = C[cidx(C_PH + 2, p)];
	cx<R> u = cfma(oxy, b, oxx * a), v = cfma(oyy, b, oxy * a);
	a = u;
	b = v;
}

// x pass of the shift operator for every slot (q = 0 slots included: their weights are
// exactly 0/1/0/0 and the pass reduces to the duplicate-column copy), optionally preceded by
// the phase operator of coefficient set CA applied at each tap: T = X(phase_A(F)).
template <typename R>
__global__ void k_shift_x(Geom G, int slot0, const ShiftParams* __restrict__ sp, const cx<R>* __restrict__ CA,
		const cx<R>* __restrict__ F, cx<R>* __restrict__ T) {
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= G.N) return;
	int s = blockIdx.y;
	int gs = slot0 + s;
	int g = gs / G.spg - slot0 / G.spg;
	int gq = (gs / G.spg) * G.Nq + (gs / 2) % G.Nq;
	const ShiftParams P = sp[gq];
	const size_t N = G.N;
	const int Nx = G.Nx;
	int ix = p % Nx, iy = p / Nx;
	const cx<R>* f = F + (size_t)s * 2 * N;
	const cx<R>* Cg = CA ? CA + (size_t)g * coef_set_size(N) : nullptr;
	cx<R> v0, v1;
	if(Nx > 3) {
		v0 = mk<R>(0, 0);
		v1 = mk<R>(0, 0);
#pragma unroll
		for(int k = 0; k < 4; k++) {
			int q = ref_wrap(ix + P.msx - 1 + k, Nx) + Nx * iy;
			cx<R> a = f[q], b = f[N + q];
			if(Cg) phase_apply(Cg, N, q, a, b);
			v0 += (R)P.wx[k] * a;
			v1 += (R)P.wx[k] * b;
		}
	}
	else {
		v0 = f[p];
		v1 = f[N + p];
		if(Cg) phase_apply(Cg, N, p, v0, v1);
	}
	T[(size_t)s * 2 * N + p] = v0;
	T[(size_t)s * 2 * N + N + p] = v1;
}

// y pass and phase factor of the shift operator, optionally followed by the phase operator
// of coefficient set CB: F = phase_B(ph * Y(T)).
template <typename R>
__global__ void k_shift_y(Geom G, int slot0, const ShiftParams* __restrict__ sp, const cx<R>* __restrict__ CB,
		const cx<R>* __restrict__ T, cx<R>* __restrict__ F) {
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= G.N) return;
	int s = blockIdx.y;
	int gs = slot0 + s;
	int g = gs / G.spg - slot0 / G.spg;
	int gq = (gs / G.spg) * G.Nq + (gs / 2) % G.Nq;
	const ShiftParams P = sp[gq];
	const size_t N = G.N;
	const int Nx = G.Nx, Ny = G.Ny;
	int ix = p % Nx, iy = p / Nx;
	const cx<R>* t = T + (size_t)s * 2 * N;
	cx<R> ph = mk<R>((R)P.ph_re, (R)P.ph_im);
	cx<R> v0, v1;
	if(Ny > 3) {
		v0 = mk<R>(0, 0);
		v1 = mk<R>(0, 0);
#pragma unroll
		for(int k = 0; k < 4; k++) {
			int q = ix + Nx * ref_wrap(iy + P.msy - 1 + k, Ny);
			v0 += (R)P.wy[k] * t[q];
			v1 += (R)P.wy[k] * t[N + q];
		}
	}
	else {
		v0 = t[p];
		v1 = t[N + p];
	}
	v0 = v0 * ph;
	v1 = v1 * ph;
	if(CB) phase_apply(CB + (size_t)g * coef_set_size(N), N, p, v0, v1);
	F[(size_t)s * 2 * N + p] = v0;
	F[(size_t)s * 2 * N + N + p] = v1;
}

// Whole transition between two slabs in one pass (replaces shift_x(A), shift_y, shift_x,
// shift_y(B)): F_out = phase_B(ph^n * Y^n X^n (phase_A(F))), n = nshift (1 or 2). X and Y are
// the circulant cubic shifts of SimpleShiftOperator (period Nx-1 / Ny-1; they act on rows and
// columns and commute, so Y X Y X = Y Y X X). For a tile of 32 x 32 outputs of one slot the
// block stages the input window (phase_A applied) in shared memory; each thread then runs the n
// x-passes over 8 consecutive outputs of a window row in registers (the 8 + 3n inputs read once)
// into a second buffer, and the n y-passes over 4 consecutive rows of an output column, and
// writes the tile. Indices wrap with i mod (N-1), which equals the
// reference's wrap rule for every index above -(N-1) (the composition of two wrapped passes
// then also reduces to one mod); a slot whose integer shift reaches -(N-2) or below takes the
// exact per-point path instead. The duplicate row and column of F are never read, as in the
// separate passes.
constexpr int SHT = 32;  // tile edge

__device__ __forceinline__ int pmod(int i, int n) {
	int r = i % n;
	return r < 0 ? r + n : r;
}

template <typename R>
__device__ __forceinline__ void tap_in(const cx<R>* f, const cx<R>* Ca, size_t N, int q, cx<R>& a, cx<R>& b) {
	a = f[q];
	b = f[N + q];
	if(Ca) phase_apply(Ca, N, q, a, b);
}

// Exact composition with the reference's wrap rule, one output point (rarely used).
template <typename R>
__device__ void shift_point_exact(const Geom& G, const ShiftParams& P, const cx<R>* f, const cx<R>* Ca, int nsh,
		int ix, int iy, cx<R>& o0, cx<R>& o1) {
	const size_t N = G.N;
	const int Nx = G.Nx, Ny = G.Ny;
	const bool ax = Nx > 3, ay = Ny > 3;
	auto xrow = [&](int r, int x, cx<R>& a, cx<R>& b) {  // X^n of row r at column x
		if(!ax) { tap_in(f, Ca, N, x + Nx * r, a, b); return; }
		a = b = mk<R>(0, 0);
		for(int k1 = 0; k1 < 4; k1++) {
			int j = ref_wrap(x + P.msx - 1 + k1, Nx);
			cx<R> u0 = mk<R>(0, 0), u1 = mk<R>(0, 0);
			if(nsh == 2) {
				for(int k0 = 0; k0 < 4; k0++) {
					cx<R> t0, t1;
					tap_in(f, Ca, N, ref_wrap(j + P.msx - 1 + k0, Nx) + Nx * r, t0, t1);
					u0 += (R)P.wx[k0] * t0;
					u1 += (R)P.wx[k0] * t1;
				}
			}
			else tap_in(f, Ca, N, j + Nx * r, u0, u1);
			a += (R)P.wx[k1] * u0;
			b += (R)P.wx[k1] * u1;
		}
	};
	if(!ay) { xrow(iy, ix, o0, o1); return; }
	o0 = o1 = mk<R>(0, 0);
	for(int l1 = 0; l1 < 4; l1++) {
		int r1 = ref_wrap(iy + P.msy - 1 + l1, Ny);
		cx<R> u0 = mk<R>(0, 0), u1 = mk<R>(0, 0);
		if(nsh == 2) {
			for(int l0 = 0; l0 < 4; l0++) {
				cx<R> t0, t1;
				xrow(ref_wrap(r1 + P.msy - 1 + l0, Ny), ix, t0, t1);
				u0 += (R)P.wy[l0] * t0;
				u1 += (R)P.wy[l0] * t1;
			}
		}
		else xrow(r1, ix, u0, u1);
		o0 += (R)P.wy[l1] * u0;
		o1 += (R)P.wy[l1] * u1;
	}
}

template <typename R>
__global__ void __launch_bounds__(256) k_shift_fused(Geom G, int slot0, const ShiftParams* __restrict__ sp,
		const cx<R>* __restrict__ CA, const cx<R>* __restrict__ CB, int nsh, const cx<R>* __restrict__ F,
		cx<R>* __restrict__ Fo) {
	extern __shared__ unsigned char smem_raw[];
	const int s = blockIdx.z;
	const int gs = slot0 + s;
	const int g = gs / G.spg - slot0 / G.spg;
	const int gq = (gs / G.spg) * G.Nq + (gs / 2) % G.Nq;
	const ShiftParams& P = sp[gq];
	const ShiftW<R> W(P);
	const size_t N = G.N;
	const int Nx = G.Nx, Ny = G.Ny;
	const bool ax = Nx > 3, ay = Ny > 3;
	const int x0 = blockIdx.x * SHT, y0 = blockIdx.y * SHT;
	const int tid = threadIdx.x;
	const cx<R>* f = F + (size_t)s * 2 * N;
	cx<R>* fo = Fo + (size_t)s * 2 * N;
	const cx<R>* Ca = CA ? CA + (size_t)g * coef_set_size(N) : nullptr;
	const cx<R>* Cb = CB ? CB + (size_t)g * coef_set_size(N) : nullptr;
	const int Px = Nx - 1, Py = Ny - 1;
	const int bx = ax ? nsh * (P.msx - 1) : 0, by = ay ? nsh * (P.msy - 1) : 0;
	const int wx = ax ? SHT + 3 * nsh : SHT, wy = ay ? SHT + 3 * nsh : SHT;
	cx<R> ph = W.ph;
	if(nsh == 2) ph = ph * ph;
	// every tap index of both passes stays above -(N-1): mod arithmetic equals the wrap rule
	const bool regular = (!ax || P.msx - 1 > -Px) && (!ay || P.msy - 1 > -Py);
	if(!regular) {
		for(int e = tid; e < SHT * SHT; e += blockDim.x) {
			int ix = x0 + e % SHT, iy = y0 + e / SHT;
			if(ix >= Nx || iy >= Ny) continue;
			cx<R> o0, o1;
			shift_point_exact(G, P, f, Ca, nsh, ix, iy, o0, o1);
			o0 = o0 * ph;
			o1 = o1 * ph;
			int p = ix + Nx * iy;
			if(Cb) phase_apply(Cb, N, p, o0, o1);
			fo[p] = o0;
			fo[N + p] = o1;
		}
		return;
	}
	// 1. input window, phase_A applied: warp w takes the window rows w, w + 8, ..., lane l the
	// columns l and l + 32; the wrapped source row and columns are computed once per row / thread
	constexpr int PA = SHT + 7, PB = SHT + 1;  // odd pitches (8-byte words): no bank conflicts
	cx<R>* A = reinterpret_cast<cx<R>*>(smem_raw);  // [2][wy][PA]: the window
	cx<R>* B = A + 2 * (SHT + 6) * PA;             // [2][wy][PB]: the window after the x-passes
	const int lane = tid % 32, warp = tid / 32, nwarp = blockDim.x / 32;
	int xc[2];
#pragma unroll
	for(int h = 0; h < 2; h++) {
		const int u = lane + 32 * h;
		xc[h] = u >= wx ? -1 : ax ? pmod(x0 + bx + u, Px) : (x0 + u < Nx ? x0 + u : -1);
	}
	for(int v = warp; v < wy; v += nwarp) {
		const int yi = ay ? pmod(y0 + by + v, Py) : (y0 + v < Ny ? y0 + v : -1);
#pragma unroll
		for(int h = 0; h < 2; h++) {
			const int u = lane + 32 * h;
			if(u < wx) {
				cx<R> a = mk<R>(0, 0), b = mk<R>(0, 0);
				if(xc[h] >= 0 && yi >= 0) tap_in(f, Ca, N, xc[h] + Nx * yi, a, b);
				A[v * PA + u] = a;
				A[(SHT + 6) * PA + v * PA + u] = b;
			}
		}
	}
	__syncthreads();
	// 2. the n x-passes of one component over 8 consecutive outputs of a window row per thread, in
	// registers (consecutive threads take consecutive rows)
	const cx<R>* Y = A;  // what the y-passes read, with its pitch
	int PY = PA;
	if(ax) {
		const int nin = 8 + 3 * nsh;
		for(int t = tid; t < 2 * 4 * wy; t += blockDim.x) {
			const int v = t % wy, r = t / wy, seg = r % 4, c = r / 4;
			const cx<R>* in = A + c * (SHT + 6) * PA + v * PA + seg * 8;
			cx<R> w[14];
#pragma unroll
			for(int k = 0; k < 14; k++) w[k] = k < nin ? in[k] : mk<R>(0, 0);
			// first pass: 8 + 3 (n - 1) values, second pass (n = 2): 8
#pragma unroll
			for(int k = 0; k < 11; k++) w[k] = W.wx[0] * w[k] + W.wx[1] * w[k + 1] + W.wx[2] * w[k + 2] + W.wx[3] * w[k + 3];
			if(nsh == 2) {
#pragma unroll
				for(int k = 0; k < 8; k++) w[k] = W.wx[0] * w[k] + W.wx[1] * w[k + 1] + W.wx[2] * w[k + 2] + W.wx[3] * w[k + 3];
			}
			cx<R>* out = B + c * (SHT + 6) * PB + v * PB + seg * 8;
#pragma unroll
			for(int k = 0; k < 8; k++) out[k] = w[k];
		}
		__syncthreads();
		Y = B;
		PY = PB;
	}
	// 3. the n y-passes over 4 consecutive output rows of one column per thread (both components),
	// then the phase factor, phase_B and the store (consecutive threads take consecutive columns)
	for(int t = tid; t < SHT * (SHT / 4); t += blockDim.x) {
		const int u = t % SHT, seg = t / SHT;
		const int ix = x0 + u;
		cx<R> o[2][4];
#pragma unroll
		for(int c = 0; c < 2; c++) {
			const cx<R>* in = Y + c * (SHT + 6) * PY + seg * 4 * PY + u;
			if(ay) {
				const int nin = 4 + 3 * nsh;
				cx<R> w[10];
#pragma unroll
				for(int k = 0; k < 10; k++) w[k] = k < nin ? in[k * PY] : mk<R>(0, 0);
#pragma unroll
				for(int k = 0; k < 7; k++) w[k] = W.wy[0] * w[k] + W.wy[1] * w[k + 1] + W.wy[2] * w[k + 2] + W.wy[3] * w[k + 3];
				if(nsh == 2) {
#pragma unroll
					for(int k = 0; k < 4; k++) w[k] = W.wy[0] * w[k] + W.wy[1] * w[k + 1] + W.wy[2] * w[k + 2] + W.wy[3] * w[k + 3];
				}
#pragma unroll
				for(int k = 0; k < 4; k++) o[c][k] = w[k];
			}
			else {
#pragma unroll
				for(int k = 0; k < 4; k++) o[c][k] = in[k * PY];
			}
		}
		if(ix >= Nx) continue;
#pragma unroll
		for(int k = 0; k < 4; k++) {
			const int iy = y0 + seg * 4 + k;
			if(iy < Ny) {
				cx<R> o0 = o[0][k] * ph, o1 = o[1][k] * ph;
				const int p = ix + Nx * iy;
				if(Cb) phase_apply(Cb, N, p, o0, o1);
				fo[p] = o0;
				fo[N + p] = o1;
			}
		}
	}
}

// All slots at q = 0: phase_A, then the shift operator's duplicate-border copy (column 0 ->
// column Nx-1, then row 0 -> row Ny-1), then phase_B, in one in-place pass. The thread of a
// source point also writes the border points copied from it, so no thread reads a value
// another thread writes.
template <typename R>
__global__ void k_phase_sync(Geom G, int slot0, const cx<R>* __restrict__ CA, const cx<R>* __restrict__ CB,
		cx<R>* F) {
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= G.N) return;
	int s = blockIdx.y;
	int g = (slot0 + s) / G.spg - slot0 / G.spg;
	const size_t N = G.N;
	const int Nx = G.Nx, Ny = G.Ny;
	const bool ax = Nx > 3, ay = Ny > 3;
	int ix = p % Nx, iy = p / Nx;
	if((ax && ix == Nx - 1) || (ay && iy == Ny - 1)) return;
	cx<R>* f = F + (size_t)s * 2 * N;
	const cx<R>* Ca = CA ? CA + (size_t)g * coef_set_size(N) : nullptr;
	const cx<R>* Cb = CB ? CB + (size_t)g * coef_set_size(N) : nullptr;
	cx<R> u0 = f[p], u1 = f[N + p];
	if(Ca) phase_apply(Ca, N, p, u0, u1);
	auto put = [&](int d) {
		cx<R> a = u0, b = u1;
		if(Cb) phase_apply(Cb, N, d, a, b);
		f[d] = a;
		f[N + d] = b;
	};
	put(p);
	if(ax && ix == 0) put((Nx - 1) + Nx * iy);
	if(ay && iy == 0) put(ix + Nx * (Ny - 1));
	if(ax && ay && ix == 0 && iy == 0) put((Nx - 1) + Nx * (Ny - 1));
}

// Entrance field: beam profile with polarisation angle pi/2*pol (BPMIteration.cpp:87-109,
// BeamProfile.cpp:17-39) followed by the input Fresnel operator (FresnelOperator.cpp:16-38)
// built on sqrt(eps_tr) at iz = 0.
template <typename R>
__global__ void k_init_fields(Geom G, int slot0, const GroupParams* __restrict__ gps, const R* __restrict__ Q0,
		int beam_type, double waist, double dx, double dy, double cpol1, double spol1, cx<R>* F) {
	// arithmetic in the plan's precision (FP32 mode: FP32, within its error budget)
	using T = R;
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= G.N) return;
	int s = blockIdx.y;
	int N = G.N, Nx = G.Nx, Ny = G.Ny;
	int gs = slot0 + s;
	int g = gs / G.spg - slot0 / G.spg;
	int pol = gs % 2;
	// polarisation (cos, sin)(pi/2 * pol); the pol = 1 values come from the host's libm
	const T cth = pol ? (T)cpol1 : (T)1, sth = pol ? (T)spol1 : (T)0;
	T amp = 1;
	if(beam_type == 1) {
		const T x = (T)(((p % Nx) - (Nx - 1) / 2.) * dx), y = (T)(((p / Nx) - (Ny - 1) / 2.) * dy), w = (T)waist;
		amp = exp(-(x * x + y * y) / (2 * w * w));
	}
	const T ex = cth * amp, ey = sth * amp;
	const R* Q = Q0 + (size_t)g * NQ * N;
	const T nxx = Q[Q_XXS * N + p], nyy = Q[Q_YYS * N + p], nxy = Q[Q_XYS * N + p];
	const T n = (T)gps[g].nin;
	const T det = (n + nxx) * (n + nyy) - nxy * nxy;
	const T a = 2 * n * (n + nyy) / det * ex - 2 * n * nxy / det * ey;
	const T b = -2 * n * nxy / det * ex + 2 * n * (n + nxx) / det * ey;
	F[(size_t)s * 2 * N + p] = mk<R>((R)a, 0);
	F[(size_t)s * 2 * N + N + p] = mk<R>((R)b, 0);
}

// Output Fresnel operator at iz = Nz-1 (FresnelOperator.cpp:45-69), in the plan's precision.
template <typename R>
__global__ void k_fresnel_out(Geom G, int slot0, const GroupParams* __restrict__ gps, const R* __restrict__ QL,
		cx<R>* F) {
	using T = R;
	int p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= G.N) return;
	int s = blockIdx.y;
	int N = G.N;
	int g = (slot0 + s) / G.spg - slot0 / G.spg;
	const R* Q = QL + (size_t)g * NQ * N;
	const T nxx = Q[Q_XXS * N + p], nyy = Q[Q_YYS * N + p], nxy = Q[Q_XYS * N + p];
	const T n = (T)gps[g].nout_fresnel;
	const T det = (n + nxx) * (n + nyy) - nxy * nxy;
	const T axx = 2 * (1 - n * (n + nyy) / det), ayy = 2 * (1 - n * (n + nxx) / det), axy = 2 * (n * nxy / det);
	cx<R>* f = F + (size_t)s * 2 * N + p;
	const cx<R> a = f[0], b = f[N];
	f[0] = axx * a + axy * b;
	f[N] = ayy * b + axy * a;
}

template <typename R>
__global__ void k_copy(size_t n, const cx<R>* __restrict__ a, cx<R>* __restrict__ b) {
	size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n) b[i] = a[i];
}

template <typename R>
__global__ void k_widen(size_t n, const cx<R>* __restrict__ a, cx<double>* __restrict__ b) {
	size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n) b[i] = cvt<double>(a[i]);
}

template <typename R>
__global__ void k_narrow(size_t n, const cx<double>* __restrict__ a, cx<R>* __restrict__ b) {
	size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n) b[i] = cvt<R>(a[i]);
}

}  // namespace nbpm
