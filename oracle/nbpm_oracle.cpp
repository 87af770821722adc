// FP64 CPU restatement of the Nemaktis bpm-solver backend path (the oracle).
//
// TEST INFRASTRUCTURE ONLY. Nothing in the nemaktis_gb300 product links, loads or calls
// this file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as the
// checker and as the timed CPU restatement of the reference.
//
// Parity status: UNPINNED against the reference binary. The reference (Eigen, FFTW,
// muParser, Boost, VTK) cannot be compiled in this environment and ships no golden
// vectors for this path, so this restatement is checked by invariants (unitarity,
// x-invariance, uniform-medium Jones retardation), by the analytic uniform-crystal
// propagator of the reference's own benchmark scripts, and its FFT against numpy.fft.
//
// Every routine below restates one function of the reference (paths relative to the
// reference project root) and keeps its index quirks:
//   BeamPropagationSolver/src/PhysicsLib/PermittivityTensorField.cpp:3-99
//   BeamPropagationSolver/src/BeamPropagationLib/BlockSparseMatrix.cpp:70-646
//   BeamPropagationSolver/src/BeamPropagationLib/ParaxialPrimaryEvolutionOperator.cpp:4-490
//   BeamPropagationSolver/src/BeamPropagationLib/PhaseEvolutionOperator.cpp:3-63
//   BeamPropagationSolver/src/BeamPropagationLib/SimpleShiftOperator.cpp:3-93, .h:24-39
//   BeamPropagationSolver/src/BeamPropagationLib/FresnelOperator.cpp:16-69
//   BeamPropagationSolver/src/BeamPropagationLib/BPMIteration.cpp:53-177
//   BeamPropagationSolver/src/PostprocessorLib/ScreenOutput.cpp:13-39,184-302
// The sparse matrices of the reference are held here as per-(block, stencil-shift, row)
// value planes; row-wise and column-wise assembly loops of the reference become per-entry
// additions with the coefficient taken at the row point or at the column point.

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef std::complex<double> cd;
const double PI_REF = 3.1415926535897932;  // PhysicsCoefficients.h:14

struct Params {
	int Nx, Ny, Nz;
	double dx, dy, dz;
	int field_dim;
	int n_woodbury;
	int beam_type;  // 0 UniformBeam, 1 GaussianBeam, 2 None
	double waist;
	int n_wavelengths;
	const double* wavelengths;
	const double* no;
	const double* ne;
	const double* ne_imag;
	const double* nhost;
	const double* nin;
	const double* nout;
	int n_q;
	const double* q;
	int n_iso;
	const double* iso_thick;
	const double* iso_index;
	double z_foc;
	double numerical_aperture;
	double nout_06;
};

// ---------------------------------------------------------------------------------------
// Permittivity tensor field, PermittivityTensorField.cpp:3-99 (12 comps per voxel).
// ---------------------------------------------------------------------------------------
struct Eps {
	int Nx, Ny, Nz;
	std::vector<double> v;
	double nref;
	double at(int ix, int iy, int iz, int c) const {
		return v[c + 12 * (ix + (size_t)Nx * (iy + (size_t)Ny * iz))];
	}
	double xx(int x, int y, int z) const { return at(x, y, z, 0); }
	double yy(int x, int y, int z) const { return at(x, y, z, 1); }
	double zz(int x, int y, int z) const { return at(x, y, z, 2); }
	double xy(int x, int y, int z) const { return at(x, y, z, 3); }
	double xz(int x, int y, int z) const { return at(x, y, z, 4); }
	double yz(int x, int y, int z) const { return at(x, y, z, 5); }
	double xx_tr(int x, int y, int z) const { return at(x, y, z, 6); }
	double yy_tr(int x, int y, int z) const { return at(x, y, z, 7); }
	double xy_tr(int x, int y, int z) const { return at(x, y, z, 8); }
	double xx_sqrt(int x, int y, int z) const { return at(x, y, z, 9); }
	double yy_sqrt(int x, int y, int z) const { return at(x, y, z, 10); }
	double xy_sqrt(int x, int y, int z) const { return at(x, y, z, 11); }
};

void build_eps(Eps& e, const Params& P, const double* lc, const unsigned char* mask,
		double no, double ne, double nhost) {
	e.Nx = P.Nx; e.Ny = P.Ny; e.Nz = P.Nz;
	size_t nv = (size_t)P.Nx * P.Ny * P.Nz;
	e.v.assign(12 * nv, 0.);
	double eps_perp = std::pow(no, 2.);
	double eps_a = std::pow(ne, 2.) - eps_perp;
	double eps_host = std::pow(nhost, 2.);
	int fd = P.field_dim;
	if(fd == 3) {
		#pragma omp parallel for
		for(long long i = 0; i < (long long)nv; i++) {
			bool m = mask ? (mask[i] != 0) : true;
			const double* n = lc + 3 * i;
			double* o = &e.v[12 * i];
			o[0] = m ? eps_perp + eps_a * std::pow(n[0], 2.) : eps_host;
			o[1] = m ? eps_perp + eps_a * std::pow(n[1], 2.) : eps_host;
			o[2] = m ? eps_perp + eps_a * std::pow(n[2], 2.) : eps_host;
			o[3] = m ? eps_a * n[0] * n[1] : 0;
			o[4] = m ? eps_a * n[0] * n[2] : 0;
			o[5] = m ? eps_a * n[1] * n[2] : 0;
		}
	}
	else {
		double eps_a_eff = 2 * eps_a / 3;
		double eps_iso = eps_perp + eps_a / 3.;
		#pragma omp parallel for
		for(long long i = 0; i < (long long)nv; i++) {
			bool m = mask ? (mask[i] != 0) : true;
			const double* Q = lc + 6 * i;
			double* o = &e.v[12 * i];
			o[0] = m ? eps_iso + eps_a_eff * Q[0] : eps_host;
			o[1] = m ? eps_iso + eps_a_eff * Q[1] : eps_host;
			o[2] = m ? eps_iso + eps_a_eff * Q[2] : eps_host;
			o[3] = m ? eps_a_eff * Q[3] : 0;
			o[4] = m ? eps_a_eff * Q[4] : 0;
			o[5] = m ? eps_a_eff * Q[5] : 0;
		}
	}
	double nref_sum = 0;
	#pragma omp parallel for reduction(+:nref_sum)
	for(long long i = 0; i < (long long)nv; i++) {
		double* o = &e.v[12 * i];
		o[6] = o[0] - std::pow(o[4], 2) / o[2];
		o[7] = o[1] - std::pow(o[5], 2) / o[2];
		o[8] = o[3] - o[4] * o[5] / o[2];
		double det = o[6] * o[7] - o[8] * o[8];
		double tr = 0.5 * (o[6] + o[7]);
		double neff;
		if(tr * tr - det < 1e-8)
			neff = std::sqrt(tr);
		else
			neff = (std::sqrt(tr + std::sqrt(tr * tr - det)) + std::sqrt(tr - std::sqrt(tr * tr - det))) / 2.;
		o[9] = neff + (o[6] - o[7]) / (4 * neff);
		o[10] = neff + (o[7] - o[6]) / (4 * neff);
		o[11] = o[8] / (2 * neff);
		nref_sum += neff;
	}
	e.nref = nref_sum / ((double)P.Nx * P.Ny * P.Nz);
}

// ---------------------------------------------------------------------------------------
// Transverse 2-component field over the (Nx,Ny) plane, layout [comp][iy][ix]
// (OpticalField.h:7-96).
// ---------------------------------------------------------------------------------------
struct Field {
	int Nx, Ny, N;
	cd* d;
	cd& operator()(int ix, int iy, int c) { return d[ix + Nx * iy + N * c]; }
	cd operator()(int ix, int iy, int c) const { return d[ix + Nx * iy + N * c]; }
};

struct OwnedField : Field {
	std::vector<cd> buf;
	OwnedField(int nx, int ny) : buf(2 * (size_t)nx * ny) { Nx = nx; Ny = ny; N = nx * ny; d = buf.data(); }
};

// ---------------------------------------------------------------------------------------
// Block sparse stencil matrices, BlockSparseMatrix.cpp:70-646. Entries live at
// (block, k, row point) where k enumerates the stencil of the diff type:
//   DX:   k = 0 mx, 1 no, 2 px          (rows ix<Nx-1, all iy; only if Nx>3)
//   DY:   k = 0 my, 1 no, 2 py          (rows iy<Ny-1, all ix; only if Ny>3)
//   DXDY: k = 0 pxpy, 1 mxpy, 2 pxmy, 3 mxmy (rows ix<Nx-1, iy<Ny-1; if Nx>3 && Ny>3)
// Column points wrap with period Nx-1 / Ny-1 (BlockSparseMatrix.cpp:87-88,278-279,470-473).
// ---------------------------------------------------------------------------------------
enum DiffType { DX = 0, DY = 1, DXDY = 2 };

inline int nshift(int t) { return t == DXDY ? 4 : 3; }

struct Mesh2 {
	int Nx, Ny, N;
	bool row_ok(int t, int ix, int iy) const {
		if(t == DX) return Nx > 3 && ix < Nx - 1;
		if(t == DY) return Ny > 3 && iy < Ny - 1;
		return Nx > 3 && Ny > 3 && ix < Nx - 1 && iy < Ny - 1;
	}
	int pxi(int ix) const { return ix == Nx - 2 ? 0 : ix + 1; }
	int mxi(int ix) const { return ix == 0 ? Nx - 2 : ix - 1; }
	int pyi(int iy) const { return iy == Ny - 2 ? 0 : iy + 1; }
	int myi(int iy) const { return iy == 0 ? Ny - 2 : iy - 1; }
	void col(int t, int k, int ix, int iy, int& cx, int& cy) const {
		if(t == DX) { cy = iy; cx = (k == 0) ? mxi(ix) : (k == 1 ? ix : pxi(ix)); }
		else if(t == DY) { cx = ix; cy = (k == 0) ? myi(iy) : (k == 1 ? iy : pyi(iy)); }
		else {
			cx = (k == 0 || k == 2) ? pxi(ix) : mxi(ix);
			cy = (k == 0 || k == 1) ? pyi(iy) : myi(iy);
		}
	}
};

template <typename T>
struct StencilMat {
	int t;
	bool present[4];
	std::vector<T> val[4][4];  // [block][k][point]
	void init(int type, const Mesh2& m, const bool (&zero_blocks)[4]) {
		t = type;
		for(int b = 0; b < 4; b++) {
			present[b] = !zero_blocks[b];
			for(int k = 0; k < 4; k++)
				val[b][k].assign(present[b] && k < nshift(t) ? m.N : 0, T(0));
		}
	}
	T& at(int b, int k, int p) { return val[b][k][p]; }
	T at(int b, int k, int p) const { return val[b][k][p]; }
};

// dst[dc] (+)= A_block * src[sc] with the reference's duplicate-row/column fix-ups
// (BlockSparseMatrix.cpp:121-153, 312-344, 510-550).
void block_vmult(const Mesh2& m, const StencilMat<cd>& A, int b, Field& dst, int dc,
		const Field& src, int sc, bool add) {
	int Nx = m.Nx, Ny = m.Ny, t = A.t;
	bool active = (t == DX) ? Nx > 3 : (t == DY) ? Ny > 3 : (Nx > 3 && Ny > 3);
	if(!active) {
		if(!add)
			for(int i = 0; i < m.N; i++) dst.d[i + m.N * dc] = 0;
		return;
	}
	int ns = nshift(t);
	#pragma omp parallel for
	for(int iy = 0; iy < Ny; iy++) {
		for(int ix = 0; ix < Nx; ix++) {
			int p = ix + Nx * iy;
			if(!m.row_ok(t, ix, iy)) {
				if(!add) dst(ix, iy, dc) = 0;
				continue;
			}
			cd s = 0;
			for(int k = 0; k < ns; k++) {
				int cx, cy;
				m.col(t, k, ix, iy, cx, cy);
				s += A.at(b, k, p) * src(cx, cy, sc);
			}
			if(add) dst(ix, iy, dc) += s;
			else dst(ix, iy, dc) = s;
		}
	}
	if(t == DX) {
		for(int iy = 0; iy < Ny; iy++) dst(Nx - 1, iy, dc) = dst(0, iy, dc);
	}
	else if(t == DY) {
		for(int ix = 0; ix < Nx; ix++) dst(ix, Ny - 1, dc) = dst(ix, 0, dc);
	}
	else {
		for(int iy = 1; iy < Ny - 1; iy++) dst(Nx - 1, iy, dc) = dst(0, iy, dc);
		dst(Nx - 1, 0, dc) = dst(0, 0, dc);
		for(int ix = 0; ix < Nx; ix++) dst(ix, Ny - 1, dc) = dst(ix, 0, dc);
	}
}

// dst[dc] = (Id + s*A_block)^-1 src[sc] on periodic lines: Thomas sweep with beta0 =
// 2*mid0 plus the Sherman-Morrison corner correction (BlockSparseMatrix.cpp:195-258 for
// x-lines, 386-449 for y-lines).
void shifted_block_vmult_inv(const Mesh2& m, const StencilMat<cd>& A, int b, cd s, Field& dst,
		int dc, const Field& src, int sc) {
	int Nx = m.Nx, Ny = m.Ny;
	bool xdir = (A.t == DX);
	int L = xdir ? Nx : Ny;       // points on a line (incl. duplicate)
	int nlines = xdir ? Ny : Nx;
	if(L <= 3) {
		for(int i = 0; i < m.N; i++) dst.d[i + m.N * dc] = src.d[i + m.N * sc];
		return;
	}
	#pragma omp parallel for
	for(int line = 0; line < nlines; line++) {
		auto P = [&](int i) { return xdir ? (i + Nx * line) : (line + Nx * i); };
		auto sup = [&](int i) { return s * A.at(b, 2, P(i)); };
		auto mid = [&](int i) { return 1. + s * A.at(b, 1, P(i)); };
		auto inf = [&](int i) { return s * A.at(b, 0, P(i)); };
		cd* D = dst.d + (size_t)m.N * dc;
		const cd* S = src.d + (size_t)m.N * sc;
		std::vector<cd> gamma(L - 2), corr(L - 1);
		cd beta = 2. * mid(0);
		D[P(0)] = S[P(0)] / beta;
		corr[0] = -0.5;
		for(int i = 1; i < L - 2; i++) {
			gamma[i - 1] = sup(i - 1) / beta;
			beta = mid(i) - inf(i) * gamma[i - 1];
			D[P(i)] = (S[P(i)] - inf(i) * D[P(i - 1)]) / beta;
			corr[i] = -inf(i) * corr[i - 1] / beta;
		}
		gamma[L - 3] = sup(L - 3) / beta;
		beta = mid(L - 2) + sup(L - 2) * inf(0) / mid(0) - inf(L - 2) * gamma[L - 3];
		D[P(L - 2)] = (S[P(L - 2)] - inf(L - 2) * D[P(L - 3)]) / beta;
		corr[L - 2] = (sup(L - 2) - inf(L - 2) * corr[L - 3]) / beta;
		for(int i = L - 2; i > 0; i--) {
			D[P(i - 1)] -= gamma[i - 1] * D[P(i)];
			corr[i - 1] -= gamma[i - 1] * corr[i];
		}
		cd frac = (D[P(0)] - inf(0) / mid(0) * D[P(L - 2)]) /
			(1. + corr[0] - inf(0) / mid(0) * corr[L - 2]);
		for(int i = 0; i < L - 1; i++) D[P(i)] -= frac * corr[i];
		D[P(L - 1)] = D[P(0)];
	}
}

// ---------------------------------------------------------------------------------------
// ParaxialPrimaryEvolutionOperator (ParaxialPrimaryEvolutionOperator.cpp:4-490).
// ---------------------------------------------------------------------------------------
struct Primary {
	Mesh2 m;
	const Eps& eps;
	double dX, dY, dZ;
	int n_wood;
	cd mu;
	StencilMat<double> D0[3], D1[3], D[3];
	StencilMat<cd> R[3];
	OwnedField tmp, tmp2;

	Primary(const Eps& e, const Params& P, double wavelength)
		: eps(e), tmp(P.Nx, P.Ny), tmp2(P.Nx, P.Ny) {
		m.Nx = P.Nx; m.Ny = P.Ny; m.N = P.Nx * P.Ny;
		double k0 = 2 * PI_REF / wavelength;
		dX = k0 * P.dx; dY = k0 * P.dy; dZ = k0 * P.dz;
		n_wood = P.n_woodbury;
		mu = cd(0, dZ / 2.);
		// D0: zero blocks DX {T,T,T,F}, DY {F,T,T,T}, DXDY {T,F,F,T} (:12-14)
		bool z0dx[4] = {true, true, true, false}, z0dy[4] = {false, true, true, true},
			zxy[4] = {true, false, false, true};
		// D1: DX {F,T,T,T}, DY {T,T,T,F}, DXDY {T,F,F,T} (:15-17)
		bool z1dx[4] = {false, true, true, true}, z1dy[4] = {true, true, true, false};
		bool full[4] = {false, false, false, false};
		D0[DX].init(DX, m, z0dx); D0[DY].init(DY, m, z0dy); D0[DXDY].init(DXDY, m, zxy);
		D1[DX].init(DX, m, z1dx); D1[DY].init(DY, m, z1dy); D1[DXDY].init(DXDY, m, zxy);
		for(int t = 0; t < 3; t++) { D[t].init(t, m, full); R[t].init(t, m, full); }
		int Nx = m.Nx, Ny = m.Ny;
		// D0 stencil values (:71-99)
		for(int iy = 0; iy < Ny; iy++) {
			for(int ix = 0; ix < Nx; ix++) {
				int p = ix + Nx * iy;
				if(iy < Ny - 1 && Ny > 3) {
					D0[DY].at(0, 0, p) = 1. / std::pow(dY, 2.);
					D0[DY].at(0, 1, p) = -2. / std::pow(dY, 2.);
					D0[DY].at(0, 2, p) = 1. / std::pow(dY, 2.);
				}
				if(iy < Ny - 1 && ix < Nx - 1 && Nx > 3 && Ny > 3) {
					for(int b : {1, 2}) {
						D0[DXDY].at(b, 0, p) = -0.25 / (dX * dY);  // pxpy
						D0[DXDY].at(b, 2, p) = 0.25 / (dX * dY);   // pxmy
						D0[DXDY].at(b, 1, p) = 0.25 / (dX * dY);   // mxpy
						D0[DXDY].at(b, 3, p) = -0.25 / (dX * dY);  // mxmy
					}
				}
				if(ix < Nx - 1 && Nx > 3) {
					D0[DX].at(3, 0, p) = 1. / std::pow(dX, 2.);
					D0[DX].at(3, 1, p) = -2. / std::pow(dX, 2.);
					D0[DX].at(3, 2, p) = 1. / std::pow(dX, 2.);
				}
			}
		}
	}

	// update_D1 (:421-490), with the x/y neighbour quirk p_px=(ix==Nx-1)?1:ix+1,
	// p_mx=(ix==0)?Nx-2:ix-1 of :428-431.
	void update_D1(int iz) {
		int Nx = m.Nx, Ny = m.Ny;
		#pragma omp parallel for
		for(int iy = 0; iy < Ny; iy++) {
			for(int ix = 0; ix < Nx; ix++) {
				int p = ix + Nx * iy;
				int pxx = (ix == Nx - 1) ? 1 : ix + 1, mxx = (ix == 0) ? Nx - 2 : ix - 1;
				int pyy = (iy == Ny - 1) ? 1 : iy + 1, myy = (iy == 0) ? Ny - 2 : iy - 1;
				double e = (1. / eps.zz(ix, iy, iz) + 1. / eps.zz(ix, iy, iz + 1)) / 2;
				double epx = 0, emx = 0, epy = 0, emy = 0;
				if(Nx > 3) {
					epx = (1. / eps.zz(pxx, iy, iz) + 1. / eps.zz(pxx, iy, iz + 1)) / 2;
					emx = (1. / eps.zz(mxx, iy, iz) + 1. / eps.zz(mxx, iy, iz + 1)) / 2;
				}
				if(Ny > 3) {
					epy = (1. / eps.zz(ix, pyy, iz) + 1. / eps.zz(ix, pyy, iz + 1)) / 2;
					emy = (1. / eps.zz(ix, myy, iz) + 1. / eps.zz(ix, myy, iz + 1)) / 2;
				}
				if(ix < Nx - 1 && Nx > 3) {
					double vm = 0.5 * (emx + e) / std::pow(dX, 2.);
					double vp = 0.5 * (epx + e) / std::pow(dX, 2.);
					D1[DX].at(0, 0, p) = vm;
					D1[DX].at(0, 2, p) = vp;
					D1[DX].at(0, 1, p) = -vm - vp;
				}
				if(ix < Nx - 1 && iy < Ny - 1 && Nx > 3 && Ny > 3) {
					double a = 0.25 * epx / (dX * dY), c = 0.25 * emx / (dX * dY);
					D1[DXDY].at(1, 0, p) = a;    // pxpy
					D1[DXDY].at(1, 3, p) = c;    // mxmy
					D1[DXDY].at(1, 1, p) = -c;   // mxpy
					D1[DXDY].at(1, 2, p) = -a;   // pxmy
					double a2 = 0.25 * epy / (dX * dY), c2 = 0.25 * emy / (dX * dY);
					D1[DXDY].at(2, 0, p) = a2;   // pxpy
					D1[DXDY].at(2, 3, p) = c2;   // mxmy
					D1[DXDY].at(2, 1, p) = -a2;  // mxpy
					D1[DXDY].at(2, 2, p) = -c2;  // pxmy
				}
				if(iy < Ny - 1 && Ny > 3) {
					double vp = 0.5 * (epy + e) / std::pow(dY, 2.);
					double vm = 0.5 * (emy + e) / std::pow(dY, 2.);
					D1[DY].at(3, 2, p) = vp;
					D1[DY].at(3, 0, p) = vm;
					D1[DY].at(3, 1, p) = -vm - vp;
				}
			}
		}
	}

	// update_D (:359-419): D = D0 + D1*K, K = z-averaged transverse permittivity taken at
	// the column point.
	void update_D(int iz) {
		int Nx = m.Nx, Ny = m.Ny;
		for(int t = 0; t < 3; t++) {
			int ns = nshift(t);
			#pragma omp parallel for
			for(int iy = 0; iy < Ny; iy++) {
				for(int ix = 0; ix < Nx; ix++) {
					if(!m.row_ok(t, ix, iy)) continue;
					int p = ix + Nx * iy;
					for(int k = 0; k < ns; k++) {
						int cx, cy;
						m.col(t, k, ix, iy, cx, cy);
						double kxx = (eps.xx_tr(cx, cy, iz) + eps.xx_tr(cx, cy, iz + 1)) / 2;
						double kyy = (eps.yy_tr(cx, cy, iz) + eps.yy_tr(cx, cy, iz + 1)) / 2;
						double kxy = (eps.xy_tr(cx, cy, iz) + eps.xy_tr(cx, cy, iz + 1)) / 2;
						for(int a = 0; a < 2; a++) {
							int bx = 2 * a, by = 2 * a + 1;
							double dxv = D0[t].present[bx] ? D0[t].at(bx, k, p) : 0.;
							double dyv = D0[t].present[by] ? D0[t].at(by, k, p) : 0.;
							if(D1[t].present[bx]) dxv += D1[t].at(bx, k, p) * kxx;
							if(D1[t].present[by]) dxv += D1[t].at(by, k, p) * kxy;
							if(D1[t].present[bx]) dyv += D1[t].at(bx, k, p) * kxy;
							if(D1[t].present[by]) dyv += D1[t].at(by, k, p) * kyy;
							D[t].at(bx, k, p) = dxv;
							D[t].at(by, k, p) = dyv;
						}
					}
				}
			}
		}
	}

	// update (:212-357): R = i*W + (D*S^-1 + S^-1*D)/4.
	void update(int iz) {
		update_D1(iz);
		update_D(iz);
		int Nx = m.Nx, Ny = m.Ny;
		auto vz = [&](int a, int x, int y) {
			// i*0.25*(eps_az/eps_zz at iz and iz+1), :233-235
			double s = (a == 0)
				? (eps.xz(x, y, iz) / eps.zz(x, y, iz) + eps.xz(x, y, iz + 1) / eps.zz(x, y, iz + 1))
				: (eps.yz(x, y, iz) / eps.zz(x, y, iz) + eps.yz(x, y, iz + 1) / eps.zz(x, y, iz + 1));
			return s * cd(0, 0.25);
		};
		auto sinv = [&](int x, int y, double& ixx, double& iyy, double& ixy) {
			double exx = (eps.xx_sqrt(x, y, iz) + eps.xx_sqrt(x, y, iz + 1)) / 2;
			double eyy = (eps.yy_sqrt(x, y, iz) + eps.yy_sqrt(x, y, iz + 1)) / 2;
			double exy = (eps.xy_sqrt(x, y, iz) + eps.xy_sqrt(x, y, iz + 1)) / 2;
			double det = exx * eyy - std::pow(exy, 2.);
			ixx = eyy / det; iyy = exx / det; ixy = -exy / det;
		};
		for(int t = 0; t < 3; t++) {
			int ns = nshift(t);
			#pragma omp parallel for
			for(int iy = 0; iy < Ny; iy++) {
				for(int ix = 0; ix < Nx; ix++) {
					if(!m.row_ok(t, ix, iy)) continue;
					int p = ix + Nx * iy;
					double rxx, ryy, rxy;
					sinv(ix, iy, rxx, ryy, rxy);
					cd va[2] = {vz(0, ix, iy), vz(1, ix, iy)};
					for(int k = 0; k < ns; k++) {
						int cx, cy;
						m.col(t, k, ix, iy, cx, cy);
						cd r[4] = {0, 0, 0, 0};
						// walk-off: row-wise i/2*v_a*d_b (:237-249) then column-wise
						// i/2*d_a*v_b (:251-263); d_x (resp. d_y) only lives in DX (DY)
						// and has no centre entry.
						if(t != DXDY && k != 1) {
							double dd = (t == DX)
								? ((k == 0) ? -0.5 / dX : 0.5 / dX)
								: ((k == 0) ? -0.5 / dY : 0.5 / dY);
							cd vb[2] = {vz(0, cx, cy), vz(1, cx, cy)};
							int bcomp = (t == DX) ? 0 : 1;
							for(int a = 0; a < 2; a++) r[2 * a + bcomp] += dd * va[a];
							for(int b = 0; b < 2; b++) r[2 * bcomp + b] += dd * vb[b];
						}
						// D*S^-1 column-wise with S^-1 at the column point (:266-311)
						double cxx, cyy, cxy;
						sinv(cx, cy, cxx, cyy, cxy);
						for(int a = 0; a < 2; a++) {
							double dax = D[t].at(2 * a, k, p), day = D[t].at(2 * a + 1, k, p);
							r[2 * a] += 0.25 * dax * cxx;
							r[2 * a] += 0.25 * day * cxy;
							r[2 * a + 1] += 0.25 * dax * cxy;
							r[2 * a + 1] += 0.25 * day * cyy;
						}
						// S^-1*D row-wise with S^-1 at the row point (:312-356)
						for(int b = 0; b < 2; b++) {
							double dxb = D[t].at(b, k, p), dyb = D[t].at(2 + b, k, p);
							r[b] += 0.25 * rxx * dxb;
							r[b] += 0.25 * rxy * dyb;
							r[2 + b] += 0.25 * rxy * dxb;
							r[2 + b] += 0.25 * ryy * dyb;
						}
						for(int b = 0; b < 4; b++) R[t].at(b, k, p) = r[b];
					}
				}
			}
		}
	}

	void apply(Field& f) {
		// :153-207
		auto& Rdx = R[DX]; auto& Rdy = R[DY]; auto& Rxy = R[DXDY];
		Field& t = tmp; Field& t2 = tmp2;
		auto axpy_mu = [&](Field& dst, const Field& src) {
			for(int i = 0; i < 2 * m.N; i++) dst.d[i] += mu * src.d[i];
		};
		// Forward y-step
		block_vmult(m, Rdy, 0, t, 0, f, 0, false);
		block_vmult(m, Rdy, 1, t, 0, f, 1, true);
		block_vmult(m, Rdy, 3, t, 1, f, 1, false);
		block_vmult(m, Rxy, 3, t, 1, f, 1, true);
		block_vmult(m, Rdy, 2, t, 1, f, 0, true);
		block_vmult(m, Rxy, 2, t, 1, f, 0, true);
		axpy_mu(f, t);
		// Backward x-step
		shifted_block_vmult_inv(m, Rdx, 0, -mu, t, 0, f, 0);
		shifted_block_vmult_inv(m, Rdx, 3, -mu, t, 1, f, 1);
		std::memcpy(f.d, t.d, sizeof(cd) * 2 * m.N);
		for(int it = 0; it < n_wood; it++) {
			block_vmult(m, Rdx, 1, t2, 0, t, 1, false);
			block_vmult(m, Rxy, 1, t2, 0, t, 1, true);
			block_vmult(m, Rxy, 0, t2, 0, t, 0, true);
			block_vmult(m, Rdx, 2, t2, 1, t, 0, false);
			for(int i = 0; i < 2 * m.N; i++) t2.d[i] *= mu;
			shifted_block_vmult_inv(m, Rdx, 0, -mu, t, 0, t2, 0);
			shifted_block_vmult_inv(m, Rdx, 3, -mu, t, 1, t2, 1);
			for(int i = 0; i < 2 * m.N; i++) f.d[i] += t.d[i];
		}
		// Forward x-step
		block_vmult(m, Rdx, 0, t, 0, f, 0, false);
		block_vmult(m, Rxy, 0, t, 0, f, 0, true);
		block_vmult(m, Rdx, 1, t, 0, f, 1, true);
		block_vmult(m, Rxy, 1, t, 0, f, 1, true);
		block_vmult(m, Rdx, 3, t, 1, f, 1, false);
		block_vmult(m, Rdx, 2, t, 1, f, 0, true);
		axpy_mu(f, t);
		// Backward y-step
		shifted_block_vmult_inv(m, Rdy, 0, -mu, t, 0, f, 0);
		shifted_block_vmult_inv(m, Rdy, 3, -mu, t, 1, f, 1);
		std::memcpy(f.d, t.d, sizeof(cd) * 2 * m.N);
		for(int it = 0; it < n_wood; it++) {
			block_vmult(m, Rdy, 1, t2, 0, t, 1, false);
			block_vmult(m, Rdy, 2, t2, 1, t, 0, false);
			block_vmult(m, Rxy, 2, t2, 1, t, 0, true);
			block_vmult(m, Rxy, 3, t2, 1, t, 1, true);
			for(int i = 0; i < 2 * m.N; i++) t2.d[i] *= mu;
			shifted_block_vmult_inv(m, Rdy, 0, -mu, t, 0, t2, 0);
			shifted_block_vmult_inv(m, Rdy, 3, -mu, t, 1, t2, 1);
			for(int i = 0; i < 2 * m.N; i++) f.d[i] += t.d[i];
		}
	}
};

// ---------------------------------------------------------------------------------------
// PhaseEvolutionOperator (PhaseEvolutionOperator.cpp:3-63).
// ---------------------------------------------------------------------------------------
struct Phase {
	int Nx, Ny;
	const Eps& eps;
	const double* w;  // interp weights, 2 per (voxel of the first Nz-1 planes)
	double dZ, no;
	cd absorp;
	std::vector<cd> oxx, oyy, oxy;
	Phase(const Eps& e, const Params& P, const double* wts, double wavelength, double no_, double ne_, double nei)
		: Nx(P.Nx), Ny(P.Ny), eps(e), w(wts), no(no_) {
		dZ = 2 * PI_REF / wavelength * P.dz;
		absorp = cd(1, nei / (ne_ - no));
		oxx.resize(Nx * Ny); oyy.resize(Nx * Ny); oxy.resize(Nx * Ny);
	}
	void update(int iz) {
		const cd I(0, 1);
		#pragma omp parallel for
		for(int iy = 0; iy < Ny; iy++) {
			for(int ix = 0; ix < Nx; ix++) {
				size_t vi = ix + (size_t)Nx * (iy + (size_t)Ny * iz);
				double w0 = w[2 * vi], w1 = w[2 * vi + 1];
				double dxx = 0.5 * dZ * (w0 * eps.xx_sqrt(ix, iy, iz) + w1 * eps.xx_sqrt(ix, iy, iz + 1) - no);
				double dyy = 0.5 * dZ * (w0 * eps.yy_sqrt(ix, iy, iz) + w1 * eps.yy_sqrt(ix, iy, iz + 1) - no);
				double dxy = 0.5 * dZ * (w0 * eps.xy_sqrt(ix, iy, iz) + w1 * eps.xy_sqrt(ix, iy, iz + 1));
				double diff = (dxx - dyy) / 2.;
				double tr = (dxx + dyy) / 2.;
				double det = std::sqrt(dxy * dxy + diff * diff);
				cd sinc_det = (std::abs(det) < 1e-8) ? cd(1) : std::sin(absorp * det) / det;
				cd e = std::exp(I * absorp * tr);
				cd c = std::cos(absorp * det);
				oxx[ix + Nx * iy] = e * (c + I * diff * sinc_det);
				oyy[ix + Nx * iy] = e * (c - I * diff * sinc_det);
				oxy[ix + Nx * iy] = e * I * dxy * sinc_det;
			}
		}
	}
	void apply(Field& f) {
		#pragma omp parallel for
		for(int i = 0; i < Nx * Ny; i++) {
			cd vx = oxx[i] * f.d[i] + oxy[i] * f.d[i + Nx * Ny];
			cd vy = oxy[i] * f.d[i] + oyy[i] * f.d[i + Nx * Ny];
			f.d[i] = vx;
			f.d[i + Nx * Ny] = vy;
		}
	}
};

// ---------------------------------------------------------------------------------------
// SimpleShiftOperator (SimpleShiftOperator.cpp:3-93, wrap rule .h:24-39). The y-shift
// divides by the x spacing as in :34.
// ---------------------------------------------------------------------------------------
struct Shift {
	int Nx, Ny;
	double wx[4], wy[4];
	std::vector<int> sx[4], sy[4];
	cd phase;
	OwnedField tmp;
	int wrap(int i, int n) const {
		if(i > n - 2) return i % (n - 1);
		else if(i < 0) return i + (1 - i / (n - 1)) * (n - 1);
		return i;
	}
	Shift(const Params& P, double wavelength, double qx, double qy, double nref)
		: Nx(P.Nx), Ny(P.Ny), tmp(P.Nx, P.Ny) {
		double k0 = 2 * PI_REF / wavelength;
		double dX = k0 * P.dx, dZ = k0 * P.dz;
		phase = std::exp(-cd(0, dZ * (qx * qx + qy * qy) / (4 * nref)));
		if(Nx > 3) {
			double xs = -dZ * qx / (2 * nref * dX);
			double ms = std::floor(xs), nu = xs - ms;
			for(int ix = 0; ix < Nx; ix++)
				for(int k = 0; k < 4; k++)
					sx[k].push_back(wrap(static_cast<int>(ix + ms - 1 + k), Nx));
			wx[0] = -nu * std::pow(1 - nu, 2) / 2;
			wx[1] = (1 - nu) * (1 + nu - 3 * nu * nu / 2);
			wx[2] = nu * (1 + 4 * nu - 3 * nu * nu) / 2;
			wx[3] = -nu * nu * (1 - nu) / 2;
		}
		if(Ny > 3) {
			double ys = -dZ * qy / (2 * nref * dX);
			double ms = std::floor(ys), nu = ys - ms;
			for(int iy = 0; iy < Ny; iy++)
				for(int k = 0; k < 4; k++)
					sy[k].push_back(wrap(static_cast<int>(iy + ms - 1 + k), Ny));
			wy[0] = -nu * std::pow(1 - nu, 2) / 2;
			wy[1] = (1 - nu) * (1 + nu - 3 * nu * nu / 2);
			wy[2] = nu * (1 + 4 * nu - 3 * nu * nu) / 2;
			wy[3] = -nu * nu * (1 - nu) / 2;
		}
	}
	void apply(Field& f) {
		Field& t = tmp;
		if(Nx > 3) {
			#pragma omp parallel for
			for(int iy = 0; iy < Ny; iy++)
				for(int c = 0; c < 2; c++)
					for(int ix = 0; ix < Nx; ix++) {
						cd v = 0;
						for(int k = 0; k < 4; k++) v += wx[k] * f(sx[k][ix], iy, c);
						t(ix, iy, c) = v;
					}
		}
		else std::memcpy(t.d, f.d, sizeof(cd) * 2 * Nx * Ny);
		if(Ny > 3) {
			#pragma omp parallel for
			for(int ix = 0; ix < Nx; ix++)
				for(int c = 0; c < 2; c++)
					for(int iy = 0; iy < Ny; iy++) {
						cd v = 0;
						for(int k = 0; k < 4; k++) v += wy[k] * t(ix, sy[k][iy], c);
						f(ix, iy, c) = v;
					}
		}
		else std::memcpy(f.d, t.d, sizeof(cd) * 2 * Nx * Ny);
		for(int i = 0; i < 2 * Nx * Ny; i++) f.d[i] *= phase;
	}
};

// Fresnel operators (FresnelOperator.cpp:16-38 input, :45-69 output).
void fresnel_in(const Eps& e, double n, Field& f) {
	#pragma omp parallel for
	for(int i = 0; i < f.N; i++) {
		int ix = i % f.Nx, iy = i / f.Nx;
		double nxx = e.xx_sqrt(ix, iy, 0), nyy = e.yy_sqrt(ix, iy, 0), nxy = e.xy_sqrt(ix, iy, 0);
		double det = (n + nxx) * (n + nyy) - nxy * nxy;
		cd a = f.d[i], b = f.d[i + f.N];
		f.d[i] = 2 * n * (n + nyy) / det * a - 2 * n * nxy / det * b;
		f.d[i + f.N] = -2 * n * nxy / det * a + 2 * n * (n + nxx) / det * b;
	}
}
void fresnel_out(const Eps& e, double n, Field& f) {
	int z = e.Nz - 1;
	#pragma omp parallel for
	for(int i = 0; i < f.N; i++) {
		int ix = i % f.Nx, iy = i / f.Nx;
		double nxx = e.xx_sqrt(ix, iy, z), nyy = e.yy_sqrt(ix, iy, z), nxy = e.xy_sqrt(ix, iy, z);
		double det = (n + nxx) * (n + nyy) - nxy * nxy;
		cd a = f.d[i], b = f.d[i + f.N];
		f.d[i] = 2. * ((1. - n * (n + nyy) / det) * a + n * nxy / det * b);
		f.d[i + f.N] = 2. * ((1. - n * (n + nxx) / det) * b + n * nxy / det * a);
	}
}

// ---------------------------------------------------------------------------------------
// Mixed-radix DFT (unnormalised, sign -1 forward / +1 backward), the transform that
// fftw_plan_many_dft computes in OpticalFieldCollection.cpp:62-71. Decimation in time on
// the smallest prime factor; twiddles from std::cos/std::sin in FP64.
// ---------------------------------------------------------------------------------------
cd twiddle(long long num, long long n, int sign) {
	long long r = num % n;
	double a = 2 * PI_REF * (double)r / (double)n;
	return cd(std::cos(a), sign * std::sin(a));
}
void dft_rec(const cd* in, long long istride, cd* out, int n, int sign, cd* scratch) {
	if(n == 1) { out[0] = in[0]; return; }
	int p = 2;
	while(n % p) { p++; if(p * p > n) { p = n; break; } }
	int mm = n / p;
	for(int r = 0; r < p; r++)
		dft_rec(in + r * istride, istride * p, scratch + r * mm, mm, sign, out);
	std::vector<cd> t(p);
	for(int k = 0; k < mm; k++) {
		for(int r = 0; r < p; r++) t[r] = scratch[r * mm + k] * twiddle((long long)r * k, n, sign);
		for(int s = 0; s < p; s++) {
			cd acc = 0;
			for(int r = 0; r < p; r++) acc += t[r] * twiddle((long long)r * s, p, sign);
			out[k + mm * s] = acc;
		}
	}
}
void fft_line(cd* data, int n, long long stride, int sign) {
	std::vector<cd> in(n), out(n), scr(n);
	for(int i = 0; i < n; i++) in[i] = data[i * stride];
	dft_rec(in.data(), 1, out.data(), n, sign, scr.data());
	for(int i = 0; i < n; i++) data[i * stride] = out[i];
}
void fft2(cd* plane, int Nx, int Ny, int sign) {
	#pragma omp parallel for
	for(int iy = 0; iy < Ny; iy++) fft_line(plane + (size_t)Nx * iy, Nx, 1, sign);
	#pragma omp parallel for
	for(int ix = 0; ix < Nx; ix++) fft_line(plane + ix, Ny, Nx, sign);
}

// ScreenOutput::assemble_fourier_filter (ScreenOutput.cpp:226-302), with the |q0| quirk of
// :252 (q0_sqr is the norm, not its square).
void fourier_filter(const Params& P, double wavelength, double qx0, double qy0,
		const std::vector<double>& layer_n, double z_foc, std::vector<cd>& F /*4 per point*/) {
	int Nx = P.Nx, Ny = P.Ny;
	F.assign(4 * (size_t)Nx * Ny, 0.);
	double k0 = 2 * PI_REF / wavelength;
	double n_out = layer_n.back();
	int nl = P.n_iso;
	#pragma omp parallel for
	for(int iy = 0; iy < Ny; iy++) {
		for(int ix = 0; ix < Nx; ix++) {
			double kx = (ix < double(Nx / 2.)) ? 2 * PI_REF * ix / (P.dx * Nx) : -2 * PI_REF * (Nx - ix) / (P.dx * Nx);
			double ky = (iy < double(Ny / 2.)) ? 2 * PI_REF * iy / (P.dy * Ny) : -2 * PI_REF * (Ny - iy) / (P.dy * Ny);
			double q0 = kx / k0 + qx0, q1 = ky / k0 + qy0;
			double qn = std::sqrt(q0 * q0 + q1 * q1);
			double qn2 = std::pow(qn, 2);
			double q0s = std::sqrt(std::pow(qx0, 2) + std::pow(qy0, 2));
			cd* out = &F[4 * (ix + (size_t)Nx * iy)];
			if(!(qn < P.numerical_aperture)) continue;
			cd T[4][4];
			for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) T[a][b] = (a == b) ? 1. : 0.;
			for(int p = 0; p < nl; p++) {
				double np = layer_n[p], nn = layer_n[p + 1];
				double neff = std::sqrt(np * np - qn2), nneff = std::sqrt(nn * nn - qn2);
				double im[2][2] = {{neff + q0 * q0 / neff, q0 * q1 / neff}, {q0 * q1 / neff, neff + q1 * q1 / neff}};
				double ni[2][2] = {{(1 - std::pow(q0 / nn, 2)) / nneff, -q0 * q1 / (nn * nn * nneff)},
					{-q0 * q1 / (nn * nn * nneff), (1 - std::pow(q1 / nn, 2)) / nneff}};
				double tp[2][2], tm[2][2];
				for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) {
					double s = ni[a][0] * im[0][b] + ni[a][1] * im[1][b];
					tp[a][b] = 0.5 * ((a == b ? 1. : 0.) + s);
				}
				for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) tm[a][b] = (a == b ? 1. : 0.) - tp[a][b];
				cd g = std::exp(cd(0, (neff - std::sqrt(np * np - q0s)) * k0 * P.iso_thick[p]));
				cd L[4][4];
				for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) {
					L[a][b] = tp[a][b] * g;
					L[a][b + 2] = tm[a][b] * std::conj(g);
					L[a + 2][b] = tm[a][b] * g;
					L[a + 2][b + 2] = tp[a][b] * std::conj(g);
				}
				cd N2[4][4];
				for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) {
					cd s = 0;
					for(int c = 0; c < 4; c++) s += L[a][c] * T[c][b];
					N2[a][b] = s;
				}
				for(int a = 0; a < 4; a++) for(int b = 0; b < 4; b++) T[a][b] = N2[a][b];
			}
			cd det = T[2][2] * T[3][3] - T[2][3] * T[3][2];
			cd tmp[2][2] = {{T[3][3] / det, -T[2][3] / det}, {-T[3][2] / det, T[2][2] / det}};
			cd M[2][2];
			for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) {
				cd s = 0;
				for(int c = 0; c < 2; c++) for(int d = 0; d < 2; d++) s += T[a][c + 2] * tmp[c][d] * T[d + 2][b];
				M[a][b] = T[a][b] - s;
			}
			cd ph = std::exp(cd(0, (std::sqrt(n_out * n_out - qn2) - std::sqrt(n_out * n_out - q0s)) * k0 * z_foc));
			for(int a = 0; a < 2; a++) for(int b = 0; b < 2; b++) out[2 * a + b] = M[a][b] * ph;
		}
	}
}

void screen_output(const Params& P, cd* E) {
	int Nx = P.Nx, Ny = P.Ny, N = Nx * Ny, Nq = P.n_q;
	// ScreenOutput ctor (:13-39): z_foc -= sum_p t_p * nout(0.6) / n_p
	std::vector<double> layer_n(P.iso_index, P.iso_index + P.n_iso);
	layer_n.push_back(P.nout_06);
	double z_foc = P.z_foc;
	for(int i = 0; i < P.n_iso; i++) z_foc -= P.iso_thick[i] * P.nout_06 / layer_n[i];
	std::vector<cd> F;
	for(int w = 0; w < P.n_wavelengths; w++) {
		layer_n.back() = P.nout[w];
		cd* base = E + (size_t)w * 4 * Nq * N;
		for(int pl = 0; pl < 4 * Nq; pl++) fft2(base + (size_t)pl * N, Nx, Ny, -1);
		for(int q = 0; q < Nq; q++) {
			fourier_filter(P, P.wavelengths[w], P.q[2 * q], P.q[2 * q + 1], layer_n, z_foc, F);
			for(int pol = 0; pol < 2; pol++) {
				cd* f = base + (size_t)(pol + 2 * q) * 2 * N;
				#pragma omp parallel for
				for(int i = 0; i < N; i++) {
					cd a = f[i], b = f[i + N];
					cd t0 = F[4 * i] * a + F[4 * i + 1] * b;
					cd t1 = F[4 * i + 2] * a + F[4 * i + 3] * b;
					f[i] = t0 / double(N);
					f[i + N] = t1 / double(N);
				}
			}
		}
		for(int pl = 0; pl < 4 * Nq; pl++) fft2(base + (size_t)pl * N, Nx, Ny, +1);
	}
}

// BPMIteration::propagate_fields (BPMIteration.cpp:53-177). With bulk non-null, the fields of
// every transverse plane are recorded as the bulk output does (BPMIteration.cpp:111-121,
// 153-168: the entrance plane after the input Fresnel operator, then plane iz+1 after each
// slab, before the output Fresnel operator), as bulk[slot][iz][comp][iy][ix].
void propagate(const Params& P, const double* lc, const unsigned char* mask, const double* w, cd* E, cd* bulk) {
	int Nx = P.Nx, Ny = P.Ny, N = Nx * Ny, Nq = P.n_q;
	for(int wi = 0; wi < P.n_wavelengths; wi++) {
		double lam = P.wavelengths[wi];
		Eps eps;
		build_eps(eps, P, lc, mask, P.no[wi], P.ne[wi], P.nhost[wi]);
		Primary prim(eps, P, lam);
		Phase phase(eps, P, w, lam, P.no[wi], P.ne[wi], P.ne_imag[wi]);
		double nout_fresnel = P.n_iso > 0 ? P.iso_index[0] : P.nout[wi];
		std::vector<Shift*> shifts;
		for(int q = 0; q < Nq; q++) shifts.push_back(new Shift(P, lam, P.q[2 * q], P.q[2 * q + 1], eps.nref));
		auto field = [&](int q, int pol) {
			Field f; f.Nx = Nx; f.Ny = Ny; f.N = N;
			f.d = E + (size_t)(pol + 2 * (q + (size_t)Nq * wi)) * 2 * N;
			return f;
		};
		for(int pol = 0; pol < 2; pol++) {
			for(int q = 0; q < Nq; q++) {
				if(P.beam_type == 2) continue;
				Field f = field(q, pol);
				double th = 0.5 * PI_REF * pol;
				for(int i = 0; i < N; i++) {
					double x = ((i % Nx) - (Nx - 1) / 2.) * P.dx;
					double y = ((i / Nx) - (Ny - 1) / 2.) * P.dy;
					if(P.beam_type == 1) {
						double g = std::exp(-(x * x + y * y) / (2 * P.waist * P.waist));
						f.d[i] = std::cos(th) * g;
						f.d[i + N] = std::sin(th) * g;
					}
					else {
						f.d[i] = std::cos(th);
						f.d[i + N] = std::sin(th);
					}
				}
				fresnel_in(eps, P.nin[wi], f);
			}
		}
		auto record = [&](int iz) {
			if(!bulk) return;
			for(int pol = 0; pol < 2; pol++)
				for(int q = 0; q < Nq; q++) {
					size_t slot = pol + 2 * (q + (size_t)Nq * wi);
					Field f = field(q, pol);
					std::copy(f.d, f.d + 2 * N, bulk + (slot * P.Nz + iz) * 2 * N);
				}
		};
		record(0);
		for(int iz = 0; iz < P.Nz - 1; iz++) {
			prim.update(iz);
			phase.update(iz);
			for(int pol = 0; pol < 2; pol++) {
				for(int q = 0; q < Nq; q++) {
					Field f = field(q, pol);
					shifts[q]->apply(f);
					phase.apply(f);
					prim.apply(f);
					phase.apply(f);
					shifts[q]->apply(f);
				}
			}
			record(iz + 1);
		}
		for(int pol = 0; pol < 2; pol++)
			for(int q = 0; q < Nq; q++) {
				Field f = field(q, pol);
				fresnel_out(eps, nout_fresnel, f);
			}
		for(auto s : shifts) delete s;
	}
}

thread_local std::string g_err;

}  // namespace

extern "C" {

struct oracle_params {
	int Nx, Ny, Nz;
	double dx, dy, dz;
	int field_dim;
	int n_woodbury;
	int beam_type;
	double waist;
	int n_wavelengths;
	const double* wavelengths;
	const double* no;
	const double* ne;
	const double* ne_imag;
	const double* nhost;
	const double* nin;
	const double* nout;
	int n_q;
	const double* q;
	int n_iso;
	const double* iso_thick;
	const double* iso_index;
	double z_foc;
	double numerical_aperture;
	double nout_06;
};

// stages: bit 0 = z-propagation (BPMIteration), bit 1 = screen filter (ScreenOutput).
// bulk (nullable): (slots, Nz, 2, Ny, Nx) complex, the fields of every plane.
int oracle_run_bulk(const oracle_params* p, const double* lc, const unsigned char* mask,
		const double* interp_w, double* E, int stages, double* bulk) {
	static_assert(sizeof(oracle_params) == sizeof(Params), "layout");
	Params P;
	std::memcpy(&P, p, sizeof(P));
	cd* Ec = reinterpret_cast<cd*>(E);
	try {
		if(stages & 1) propagate(P, lc, mask, interp_w, Ec, reinterpret_cast<cd*>(bulk));
		if(stages & 2) screen_output(P, Ec);
	}
	catch(std::exception& e) {
		g_err = e.what();
		return 1;
	}
	return 0;
}

int oracle_run(const oracle_params* p, const double* lc, const unsigned char* mask,
		const double* interp_w, double* E, int stages) {
	return oracle_run_bulk(p, lc, mask, interp_w, E, stages, nullptr);
}

// Unnormalised 1-D DFT of a contiguous complex line (sign -1 forward), for tests of the
// transform against numpy.fft.
void oracle_fft1d(double* data, int n, int sign) {
	fft_line(reinterpret_cast<cd*>(data), n, 1, sign);
}

int oracle_num_threads(void) {
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

}  // extern "C"
