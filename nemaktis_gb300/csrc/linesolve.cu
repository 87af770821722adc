// Batched periodic tridiagonal line solves as a standalone C-ABI primitive.
//
// Restates BlockSparseMatrixDX/DY::shifted_block_vmult_inv (BeamPropagationSolver/src/
// BeamPropagationLib/BlockSparseMatrix.cpp:195-258, 386-449): each line has L points of which
// the last duplicates the first (period L-1); row i of the system is
//   inf_i x_{i-1} + mid_i x_i + sup_i x_{i+1} = b_i   (indices modulo L-1),  x_{L-1} = x_0,
// solved by a Thomas sweep with beta_0 = 2*mid_0 plus the Sherman-Morrison corner correction.
// Complex FP64 throughout. One thread per line: factorisation into scratch, then solve.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/nbpm.h"
#include "cplx.cuh"

namespace nbpm {

void set_last_error(const std::string& m);

// Scratch per line element: 5 complex planes (alpha, 1/beta, w, -gamma, corr), plus 2 complex
// scalars per line (r0, 1/den). The forward pass keeps gamma in the -gamma plane and the
// forward corr in the corr plane; the backward pass overwrites them in place.
__global__ void k_pt_factor(int L, int nlines, const cx<double>* __restrict__ inf, const cx<double>* __restrict__ mid,
		const cx<double>* __restrict__ sup, long long ls_in, cx<double>* __restrict__ scr) {
	int line = blockIdx.x * blockDim.x + threadIdx.x;
	if(line >= nlines) return;
	const int n = L - 1;  // unknowns per line
	const size_t P = (size_t)nlines * n;
	cx<double>* FA = scr;
	cx<double>* FRB = FA + P;
	cx<double>* FW = FRB + P;
	cx<double>* FC = FW + P;
	cx<double>* FCOR = FC + P;
	cx<double>* LS = FCOR + P + (size_t)line * 2;
	const size_t o = (size_t)line * n;
	auto I = [&](int i) { return inf[line * ls_in + i]; };
	auto Mi = [&](int i) { return mid[line * ls_in + i]; };
	auto S = [&](int i) { return sup[line * ls_in + i]; };
	const cx<double> one = mk(1.0, 0.0);
	cx<double> beta = 2.0 * Mi(0);
	cx<double> rb = crecip(beta);
	FRB[o] = rb;
	FA[o] = mk(0.0, 0.0);
	cx<double> corr = mk(-0.5, 0.0);
	FCOR[o] = corr;
	for(int i = 1; i < n - 1; i++) {
		cx<double> gam = S(i - 1) * rb;
		FC[o + i - 1] = gam;
		beta = Mi(i) - I(i) * gam;
		rb = crecip(beta);
		FRB[o + i] = rb;
		FA[o + i] = -(I(i) * rb);
		corr = -(I(i) * corr) * rb;
		FCOR[o + i] = corr;
	}
	cx<double> gl = S(n - 2) * rb;
	FC[o + n - 2] = gl;
	beta = Mi(n - 1) + cdiv(S(n - 1) * I(0), Mi(0)) - I(n - 1) * gl;
	rb = crecip(beta);
	FRB[o + n - 1] = rb;
	FA[o + n - 1] = -(I(n - 1) * rb);
	cx<double> corr_last = (S(n - 1) - I(n - 1) * corr) * rb;
	// w_i = prod_{j<i}(-gamma_j) from the forward gammas, before they are negated
	cx<double> w = one;
	FW[o] = w;
	for(int i = 1; i < n; i++) {
		w = -(w * FC[o + i - 1]);
		FW[o + i] = w;
	}
	FCOR[o + n - 1] = corr_last;
	cx<double> cn = corr_last;
	for(int i = n - 1; i > 0; i--) {
		cx<double> g = FC[o + i - 1];
		cx<double> cv = FCOR[o + i - 1] - g * cn;
		FCOR[o + i - 1] = cv;
		FC[o + i - 1] = -g;
		cn = cv;
	}
	FC[o + n - 1] = mk(0.0, 0.0);
	cx<double> r0 = cdiv(I(0), Mi(0));
	LS[0] = r0;
	LS[1] = crecip(one + cn - r0 * corr_last);
}

__global__ void k_pt_solve(int L, int nlines, long long ls_b, const cx<double>* __restrict__ scr,
		const cx<double>* __restrict__ b, cx<double>* __restrict__ x) {
	int line = blockIdx.x * blockDim.x + threadIdx.x;
	if(line >= nlines) return;
	const int n = L - 1;
	const size_t P = (size_t)nlines * n;
	const cx<double>* FA = scr;
	const cx<double>* FRB = FA + P;
	const cx<double>* FW = FRB + P;
	const cx<double>* FC = FW + P;
	const cx<double>* FCOR = FC + P;
	const cx<double>* LS = FCOR + P + (size_t)line * 2;
	const size_t o = (size_t)line * n;
	const cx<double>* bb = b + line * ls_b;
	cx<double>* xx = x + line * ls_b;
	cx<double> d = bb[0] * FRB[o];
	cx<double> acc = d;
	xx[0] = d;
	for(int i = 1; i < n; i++) {
		d = FA[o + i] * d + bb[i] * FRB[o + i];
		acc += FW[o + i] * d;
		xx[i] = d;
	}
	cx<double> fr = (acc - LS[0] * d) * LS[1];
	cx<double> dn = d;
	cx<double> v = dn - fr * FCOR[o + n - 1];
	xx[n - 1] = v;
	for(int i = n - 1; i > 0; i--) {
		cx<double> dp = xx[i - 1] + FC[o + i - 1] * dn;
		v = dp - fr * FCOR[o + i - 1];
		xx[i - 1] = v;
		dn = dp;
	}
	xx[n] = v;  // duplicate point
}

size_t pt_scratch_elems(int L, int nlines) { return (size_t)nlines * (L - 1) * 5 + (size_t)nlines * 2; }

int pt_check(int L, int nlines, const void* a, const void* b, const void* c, const void* d, const void* e,
		std::string& err) {
	if(L < 4) { err = "line length must be >= 4 (period L-1 >= 3)"; return NBPM_ERR_ARG; }
	if(nlines < 1) { err = "nlines must be >= 1"; return NBPM_ERR_ARG; }
	if(!a || !b || !c || !d || !e) { err = "null device pointer"; return NBPM_ERR_ARG; }
	return 0;
}

int pt_run(int L, int nlines, const double* inf, const double* mid, const double* sup, const double* rhs,
		double* x, cudaStream_t st, cx<double>* scr, std::string& err) {
	const int T = 128;
	const unsigned blocks = (unsigned)((nlines + T - 1) / T);
	k_pt_factor<<<blocks, T, 0, st>>>(L, nlines, reinterpret_cast<const cx<double>*>(inf),
		reinterpret_cast<const cx<double>*>(mid), reinterpret_cast<const cx<double>*>(sup), (long long)L, scr);
	k_pt_solve<<<blocks, T, 0, st>>>(L, nlines, (long long)L, scr, reinterpret_cast<const cx<double>*>(rhs),
		reinterpret_cast<cx<double>*>(x));
	cudaError_t e = cudaGetLastError();
	if(e != cudaSuccess) { err = cudaGetErrorString(e); return NBPM_ERR_CUDA; }
	return 0;
}

}  // namespace nbpm

using namespace nbpm;


extern "C" {

int nbpm_periodic_tridiag_solve(int L, int nlines, const double* inf, const double* mid, const double* sup,
		const double* rhs, double* x, void* stream) {
	std::string err;
	int rc = pt_check(L, nlines, inf, mid, sup, rhs, x, err);
	if(rc) { set_last_error(err); return rc; }
	cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
	cx<double>* scr = nullptr;
	cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&scr), pt_scratch_elems(L, nlines) * sizeof(cx<double>), st);
	if(e != cudaSuccess) {
		set_last_error(cudaGetErrorString(e));
		return e == cudaErrorMemoryAllocation ? NBPM_ERR_MEMORY : NBPM_ERR_CUDA;
	}
	rc = pt_run(L, nlines, inf, mid, sup, rhs, x, st, scr, err);
	cudaFreeAsync(scr, st);
	if(rc) { set_last_error(err); return rc; }
	e = cudaStreamSynchronize(st);
	if(e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return NBPM_ERR_CUDA; }
	return 0;
}

}  // extern "C"
