// Launchers of the chunked line-solve kernels, one translation unit per (direction,
// precision) so the many template instances compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "bpm_kernels.cuh"
#include "solve_config.h"

namespace nbpm {

struct SolveLaunch {
	int M, KS, kind;           // chunk length, slots per thread, stencil kind (ST_*)
	bool tout = false;         // k_solve_xc: transposed, component-exchanged output (ST_WOOD_X only)
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
bool launch_solve_xw(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<R>* coef, const cx<R>* fac,
	size_t plane, const cx<double>* lsc, const cx<R>* src, cx<R>* dst, const cx<R>* ai, cx<R>* ao, const cx<R>* ai2 = nullptr);
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
// y-line solve in the x-line form (k_solve_yt): grid (columns / LT, groups * nch * 2), block 32*LT,
// shared memory LT * KS * 32 * (M + 1) complex; (M, KS) as for k_solve_xc.
template <typename R>
bool launch_solve_yt(const SolveLaunch& L, Geom G, int nch, const cx<R>* coef, const cx<R>* fac, size_t plane,
	const cx<double>* lsc, const cx<R>* src, cx<R>* dst, const cx<R>* ai, cx<R>* ao, const cx<R>* ai2);
void set_solve_smem_yt_f32(int bytes);
void set_solve_smem_yt_f64(int bytes);
// Sequential y-line solve (k_solve_yq): grid (columns / block.x, groups * nch), KS in {1, 2, 4}.
// scr receives the forward values; it must alias none of src, ai, ai2 (it may be dst or ao).
template <typename R>
bool launch_solve_yq(const SolveLaunch& L, Geom G, int nch, const cx<R>* coef, const cx<R>* fac, size_t plane,
	const cx<double>* lsc, const cx<R>* src, cx<R>* scr, cx<R>* dst, const cx<R>* ai, cx<R>* ao, const cx<R>* ai2);
void set_solve_smem_x_f32(int bytes);
void set_solve_smem_x_f64(int bytes);
void set_solve_smem_y_f32(int bytes);
void set_solve_smem_y_f64(int bytes);

}  // namespace nbpm
