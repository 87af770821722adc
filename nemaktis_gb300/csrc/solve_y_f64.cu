// Instances of the chunked y-line solve kernels, double precision.
#include "solve_dispatch.cuh"

namespace nbpm {

#define NBPM_YC(MM, KK, KD) \
	if(L.M == MM && L.KS == KK && L.kind == KD) { \
		k_solve_yc<double, MM, KD, KK><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane, lsc, \
			src, dst, ai, ao, ai2); \
		return true; \
	}
#define NBPM_YC_PAIRS(KIND) \
	NBPM_YC(2, 1, KIND) NBPM_YC(2, 2, KIND) NBPM_YC(2, 4, KIND) NBPM_YC(4, 1, KIND) NBPM_YC(4, 2, KIND) NBPM_YC(4, 4, KIND) \
	NBPM_YC(8, 1, KIND) NBPM_YC(8, 2, KIND) NBPM_YC(8, 4, KIND) NBPM_YC(16, 1, KIND) NBPM_YC(16, 2, KIND) NBPM_YC(32, 1, KIND)

template <>
bool launch_solve_yc<double>(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<double>* coef,
		const cx<double>* fac, size_t plane, const cx<double>* lsc, const cx<double>* src, cx<double>* dst,
		const cx<double>* ai, cx<double>* ao, const cx<double>* ai2) {
	if(L.block.y > 16) {  // 32 warps of 8-row chunks
		if(L.M == 8 && L.KS == 1 && L.kind == ST_EXPL_X) {
			k_solve_yc<double, 8, ST_EXPL_X, 1, 1024><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane,
				lsc, src, dst, ai, ao, ai2);
			return true;
		}
		if(L.M == 8 && L.KS == 1 && L.kind == ST_WOOD_Y) {
			k_solve_yc<double, 8, ST_WOOD_Y, 1, 1024><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane,
				lsc, src, dst, ai, ao, ai2);
			return true;
		}
		if(L.M == 8 && L.KS == 2 && L.kind == ST_EXPL_X) {
			k_solve_yc<double, 8, ST_EXPL_X, 2, 1024><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane,
				lsc, src, dst, ai, ao, ai2);
			return true;
		}
		if(L.M == 8 && L.KS == 2 && L.kind == ST_WOOD_Y) {
			k_solve_yc<double, 8, ST_WOOD_Y, 2, 1024><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane,
				lsc, src, dst, ai, ao, ai2);
			return true;
		}
		return false;
	}
	NBPM_YC_PAIRS(ST_EXPL_X)
	NBPM_YC_PAIRS(ST_WOOD_Y)
	return false;
}

#define NBPM_YA(MM, KK, KD) \
	cudaFuncSetAttribute(k_solve_yc<double, MM, KD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
#define NBPM_YA_PAIRS(KIND) \
	NBPM_YA(2, 1, KIND) NBPM_YA(2, 2, KIND) NBPM_YA(2, 4, KIND) NBPM_YA(4, 1, KIND) NBPM_YA(4, 2, KIND) NBPM_YA(4, 4, KIND) \
	NBPM_YA(8, 1, KIND) NBPM_YA(8, 2, KIND) NBPM_YA(8, 4, KIND) NBPM_YA(16, 1, KIND) NBPM_YA(16, 2, KIND) NBPM_YA(32, 1, KIND)

void set_solve_smem_y_f64(int bytes) {
	cudaFuncSetAttribute(k_solve_yc<double, 8, ST_EXPL_X, 1, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	cudaFuncSetAttribute(k_solve_yc<double, 8, ST_WOOD_Y, 1, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	cudaFuncSetAttribute(k_solve_yc<double, 8, ST_EXPL_X, 2, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	cudaFuncSetAttribute(k_solve_yc<double, 8, ST_WOOD_Y, 2, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	NBPM_YA_PAIRS(ST_EXPL_X)
	NBPM_YA_PAIRS(ST_WOOD_Y)
}

#define NBPM_YS(KK, KD) \
	if(L.KS == KK && L.kind == KD) { \
		k_solve_ys<double, KD, KK><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane, lsc, src, \
			dst, ai, ao, vbuf); \
		return true; \
	}

template <>
bool launch_solve_ys<double>(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<double>* coef,
		const cx<double>* fac, size_t plane, const cx<double>* lsc, const cx<double>* src, cx<double>* dst,
		const cx<double>* ai, cx<double>* ao, cx<double>* vbuf) {
	NBPM_YS(1, ST_EXPL_X) NBPM_YS(2, ST_EXPL_X) NBPM_YS(4, ST_EXPL_X)
	NBPM_YS(1, ST_WOOD_Y) NBPM_YS(2, ST_WOOD_Y) NBPM_YS(4, ST_WOOD_Y)
	return false;
}

#define NBPM_YQ(KK, KD) \
	if(L.KS == KK && L.kind == KD) { \
		k_solve_yq<double, KD, KK><<<L.grid, L.block, 0, L.stream>>>(G, nch, coef, fac, plane, lsc, src, scr, dst, ai, ao, \
			ai2); \
		return true; \
	}

template <>
bool launch_solve_yq<double>(const SolveLaunch& L, Geom G, int nch, const cx<double>* coef, const cx<double>* fac,
		size_t plane, const cx<double>* lsc, const cx<double>* src, cx<double>* scr, cx<double>* dst, const cx<double>* ai,
		cx<double>* ao, const cx<double>* ai2) {
	NBPM_YQ(1, ST_EXPL_X) NBPM_YQ(2, ST_EXPL_X) NBPM_YQ(4, ST_EXPL_X)
	NBPM_YQ(1, ST_WOOD_Y) NBPM_YQ(2, ST_WOOD_Y) NBPM_YQ(4, ST_WOOD_Y)
	return false;
}

#define NBPM_YT(MM, KK, KD) \
	if(L.M == MM && L.KS == KK && L.kind == KD) { \
		k_solve_yt<double, MM, KD, KK><<<L.grid, L.block, L.smem, L.stream>>>(G, nch, coef, fac, plane, lsc, src, dst, ai, ao, \
			ai2); \
		return true; \
	}
#define NBPM_YT_PAIRS(KIND) \
	NBPM_YT(2, 1, KIND) NBPM_YT(2, 2, KIND) NBPM_YT(2, 4, KIND) NBPM_YT(4, 1, KIND) NBPM_YT(4, 2, KIND) NBPM_YT(4, 4, KIND) \
	NBPM_YT(8, 1, KIND) NBPM_YT(8, 2, KIND) NBPM_YT(8, 4, KIND) NBPM_YT(16, 1, KIND) NBPM_YT(16, 2, KIND) NBPM_YT(32, 1, KIND)

template <>
bool launch_solve_yt<double>(const SolveLaunch& L, Geom G, int nch, const cx<double>* coef, const cx<double>* fac,
		size_t plane, const cx<double>* lsc, const cx<double>* src, cx<double>* dst, const cx<double>* ai, cx<double>* ao,
		const cx<double>* ai2) {
	NBPM_YT_PAIRS(ST_EXPL_X)
	NBPM_YT_PAIRS(ST_WOOD_Y)
	return false;
}

#define NBPM_YTA(MM, KK, KD) \
	cudaFuncSetAttribute(k_solve_yt<double, MM, KD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
#define NBPM_YTA_PAIRS(KIND) \
	NBPM_YTA(2, 1, KIND) NBPM_YTA(2, 2, KIND) NBPM_YTA(2, 4, KIND) NBPM_YTA(4, 1, KIND) NBPM_YTA(4, 2, KIND) NBPM_YTA(4, 4, KIND) \
	NBPM_YTA(8, 1, KIND) NBPM_YTA(8, 2, KIND) NBPM_YTA(8, 4, KIND) NBPM_YTA(16, 1, KIND) NBPM_YTA(16, 2, KIND) NBPM_YTA(32, 1, KIND)

void set_solve_smem_yt_f64(int bytes) {
	NBPM_YTA_PAIRS(ST_EXPL_X)
	NBPM_YTA_PAIRS(ST_WOOD_Y)
}

}  // namespace nbpm
