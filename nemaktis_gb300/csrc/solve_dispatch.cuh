// Launchers of the chunked line-solve kernels, one translation unit per (direction,
// precision) so the many template instances compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "bpm_kernels.cuh"

namespace nbpm {

struct SolveLaunch {
	int M, KS, kind;           // chunk length, slots per thread, stencil kind (ST_*)
	dim3 grid, block;
	size_t smem;
	cudaStream_t stream;
};

// Returns false if (M, KS) has no compiled instance. ai2 (xc / yc only): a second accumulator
// input, ao = (ai + ai2) + x.
template <typename R>
bool launch_solve_xc(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<R>* coef, const cx<R>* fac,
	size_t plane, const cx<double>* lsc, const cx<R>* src, cx<R>* dst, const cx<R>* ai, cx<R>* ao,
	const cx<R>* ai2 = nullptr);
template <typename R>
bool launch_solve_yc(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<R>* coef, const cx<R>* fac,
	size_t plane, const cx<double>* lsc, const cx<R>* src, cx<R>* dst, const cx<R>* ai, cx<R>* ao,
	const cx<R>* ai2 = nullptr);
template <typename R>
bool launch_solve_xg(const SolveLaunch& L, Geom G, int slot0, const cx<R>* coef, const cx<R>* fac, size_t plane,
	const cx<double>* lsc, const cx<R>* src, cx<R>* dst, const cx<R>* ai, cx<R>* ao);
template <typename R>
bool launch_solve_xw(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<R>* coef, const cx<R>* fac,
	size_t plane, const cx<double>* lsc, const cx<R>* src, cx<R>* dst, const cx<R>* ai, cx<R>* ao);
void set_solve_smem_xw_f32(int bytes);
void set_solve_smem_xw_f64(int bytes);
template <typename R>
bool launch_solve_xs(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<R>* coef, const cx<R>* fac,
	size_t plane, const cx<double>* lsc, const cx<R>* src, cx<R>* dst, const cx<R>* ai, cx<R>* ao);
void set_solve_smem_xs_f32(int bytes);
void set_solve_smem_xs_f64(int bytes);
template <typename R>
bool launch_solve_ys(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<R>* coef, const cx<R>* fac,
	size_t plane, const cx<double>* lsc, const cx<R>* src, cx<R>* dst, const cx<R>* ai, cx<R>* ao, cx<R>* vbuf);
void set_solve_smem_xg_f32(int bytes);
void set_solve_smem_xg_f64(int bytes);
void set_solve_smem_x_f32(int bytes);
void set_solve_smem_x_f64(int bytes);
void set_solve_smem_y_f32(int bytes);
void set_solve_smem_y_f64(int bytes);

// (M, KS) pairs with compiled instances.
inline bool solve_pair_ok(int M, int KS) {
	switch(M) {
		case 2: case 4: return KS == 1 || KS == 2 || KS == 4;
		case 8: return KS == 1 || KS == 2 || KS == 4;
		case 16: return KS == 1 || KS == 2;
		case 32: return KS == 1;
	}
	return false;
}

}  // namespace nbpm
