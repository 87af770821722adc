// Instances of the chunked x-line solve kernels, double precision.
#include "solve_dispatch.cuh"

namespace nbpm {

#define NBPM_XC(MM, KK, KD) \
	if(L.M == MM && L.KS == KK && L.kind == KD && !L.tout) { \
		k_solve_xc<double, MM, KD, KK><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane, lsc, \
			src, dst, ai, ao, ai2); \
		return true; \
	} \
	if(L.M == MM && L.KS == KK && L.kind == KD && L.tout && KD == ST_WOOD_X) { \
		k_solve_xc<double, MM, ST_WOOD_X, KK, true><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane, \
			lsc, src, dst, ai, ao, ai2); \
		return true; \
	}
#define NBPM_XC_PAIRS(KIND) \
	NBPM_XC(2, 1, KIND) NBPM_XC(2, 2, KIND) NBPM_XC(2, 4, KIND) NBPM_XC(4, 1, KIND) NBPM_XC(4, 2, KIND) NBPM_XC(4, 4, KIND) \
	NBPM_XC(8, 1, KIND) NBPM_XC(8, 2, KIND) NBPM_XC(8, 4, KIND) NBPM_XC(16, 1, KIND) NBPM_XC(16, 2, KIND) NBPM_XC(32, 1, KIND)

template <>
bool launch_solve_xc<double>(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<double>* coef,
		const cx<double>* fac, size_t plane, const cx<double>* lsc, const cx<double>* src, cx<double>* dst,
		const cx<double>* ai, cx<double>* ao, const cx<double>* ai2) {
	NBPM_XC_PAIRS(ST_EXPL_Y)
	NBPM_XC_PAIRS(ST_WOOD_X)
	return false;
}

#define NBPM_XA(MM, KK, KD) \
	cudaFuncSetAttribute(k_solve_xc<double, MM, KD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
#define NBPM_XA_PAIRS(KIND) \
	NBPM_XA(2, 1, KIND) NBPM_XA(2, 2, KIND) NBPM_XA(2, 4, KIND) NBPM_XA(4, 1, KIND) NBPM_XA(4, 2, KIND) NBPM_XA(4, 4, KIND) \
	NBPM_XA(8, 1, KIND) NBPM_XA(8, 2, KIND) NBPM_XA(8, 4, KIND) NBPM_XA(16, 1, KIND) NBPM_XA(16, 2, KIND) NBPM_XA(32, 1, KIND)

#define NBPM_XAT(MM, KK) \
	cudaFuncSetAttribute(k_solve_xc<double, MM, ST_WOOD_X, KK, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);

void set_solve_smem_x_f64(int bytes) {
	NBPM_XA_PAIRS(ST_EXPL_Y)
	NBPM_XA_PAIRS(ST_WOOD_X)
	NBPM_XAT(2, 1) NBPM_XAT(2, 2) NBPM_XAT(2, 4) NBPM_XAT(4, 1) NBPM_XAT(4, 2) NBPM_XAT(4, 4)
	NBPM_XAT(8, 1) NBPM_XAT(8, 2) NBPM_XAT(8, 4) NBPM_XAT(16, 1) NBPM_XAT(16, 2) NBPM_XAT(32, 1)
}

#define NBPM_XS(KK, KD) \
	if(L.KS == KK && L.kind == KD) { \
		k_solve_xs<double, KD, KK><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, L.M, coef, fac, plane, lsc, \
			src, dst, ai, ao); \
		return true; \
	}

template <>
bool launch_solve_xs<double>(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<double>* coef,
		const cx<double>* fac, size_t plane, const cx<double>* lsc, const cx<double>* src, cx<double>* dst,
		const cx<double>* ai, cx<double>* ao) {
	NBPM_XS(1, ST_EXPL_Y) NBPM_XS(2, ST_EXPL_Y) NBPM_XS(4, ST_EXPL_Y)
	NBPM_XS(1, ST_WOOD_X) NBPM_XS(2, ST_WOOD_X) NBPM_XS(4, ST_WOOD_X)
	return false;
}

void set_solve_smem_xs_f64(int bytes) {
#define NBPM_XSA(KK, KD) cudaFuncSetAttribute(k_solve_xs<double, KD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	NBPM_XSA(1, ST_EXPL_Y) NBPM_XSA(2, ST_EXPL_Y) NBPM_XSA(4, ST_EXPL_Y)
	NBPM_XSA(1, ST_WOOD_X) NBPM_XSA(2, ST_WOOD_X) NBPM_XSA(4, ST_WOOD_X)
}

#define NBPM_XW(KK, KD) \
	if(L.M == 8 && L.KS == KK && L.kind == KD && !L.tout) { \
		k_solve_xw<double, 8, KD, KK><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane, lsc, \
			src, dst, ai, ao, ai2); \
		return true; \
	} \
	if(L.M == 8 && L.KS == KK && L.kind == KD && L.tout && KD == ST_WOOD_X) { \
		k_solve_xw<double, 8, ST_WOOD_X, KK, true><<<L.grid, L.block, L.smem, L.stream>>>(G, slot0, nch, coef, fac, plane, \
			lsc, src, dst, ai, ao, ai2); \
		return true; \
	}

template <>
bool launch_solve_xw<double>(const SolveLaunch& L, Geom G, int slot0, int nch, const cx<double>* coef,
		const cx<double>* fac, size_t plane, const cx<double>* lsc, const cx<double>* src, cx<double>* dst,
		const cx<double>* ai, cx<double>* ao, const cx<double>* ai2) {
	NBPM_XW(1, ST_EXPL_Y) NBPM_XW(2, ST_EXPL_Y) NBPM_XW(4, ST_EXPL_Y)
	NBPM_XW(1, ST_WOOD_X) NBPM_XW(2, ST_WOOD_X) NBPM_XW(4, ST_WOOD_X)
	return false;
}

void set_solve_smem_xw_f64(int bytes) {
#define NBPM_XWA(KK, KD) cudaFuncSetAttribute(k_solve_xw<double, 8, KD, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	NBPM_XWA(1, ST_EXPL_Y) NBPM_XWA(2, ST_EXPL_Y) NBPM_XWA(4, ST_EXPL_Y)
	NBPM_XWA(1, ST_WOOD_X) NBPM_XWA(2, ST_WOOD_X) NBPM_XWA(4, ST_WOOD_X)
	cudaFuncSetAttribute(k_solve_xw<double, 8, ST_WOOD_X, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	cudaFuncSetAttribute(k_solve_xw<double, 8, ST_WOOD_X, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
	cudaFuncSetAttribute(k_solve_xw<double, 8, ST_WOOD_X, 4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace nbpm
