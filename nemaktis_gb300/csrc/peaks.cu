// FMA throughput of the GPU in FP32 and FP64 (the denominators of the compute rooflines of
// the FP64 plain path and of the compute-heavy kernels). Each thread runs independent FMA
// chains in registers; the result is written so the compiler keeps the work.
#include <cuda_runtime.h>

#include <string>

#include "../../include/nbpm.h"

namespace nbpm {

void set_last_error(const std::string& m);

template <typename T, int CHAINS>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T a, T b, T* out) {
	T x[CHAINS];
#pragma unroll
	for(int c = 0; c < CHAINS; c++) x[c] = (T)(threadIdx.x + c) * (T)1e-3;
	for(int i = 0; i < iters; i++) {
#pragma unroll
		for(int c = 0; c < CHAINS; c++) x[c] = fma(x[c], a, b);
	}
	T s = 0;
#pragma unroll
	for(int c = 0; c < CHAINS; c++) s += x[c];
	if(s == (T)12345.678) out[0] = s;  // practically never taken; keeps the chains live
}

template <typename T>
static int run_peak(double* tflops) {
	int dev = 0, sms = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if(e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	T* out = nullptr;
	if(e == cudaSuccess) e = cudaMalloc(&out, sizeof(T));
	cudaEvent_t a = nullptr, b = nullptr;
	if(e == cudaSuccess) e = cudaEventCreate(&a);
	if(e == cudaSuccess) e = cudaEventCreate(&b);
	const int threads = 256, blocks = sms * 8, iters = sizeof(T) == 8 ? 2048 : 16384;
	constexpr int CH = 8;
	float ms = 0;
	if(e == cudaSuccess) {
		k_fma_peak<T, CH><<<blocks, threads>>>(16, (T)0.999, (T)1e-4, out);  // warm-up
		cudaEventRecord(a);
		k_fma_peak<T, CH><<<blocks, threads>>>(iters, (T)0.999, (T)1e-4, out);
		cudaEventRecord(b);
		e = cudaEventSynchronize(b);
	}
	if(e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
	if(a) cudaEventDestroy(a);
	if(b) cudaEventDestroy(b);
	if(out) cudaFree(out);
	if(e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return NBPM_ERR_CUDA; }
	double flops = 2.0 * (double)blocks * threads * iters * CH;
	*tflops = flops / (ms * 1e-3) / 1e12;
	return 0;
}

}  // namespace nbpm

extern "C" int nbpm_fma_peak(int precision, double* tflops) {
	if(!tflops) { nbpm::set_last_error("null argument"); return NBPM_ERR_ARG; }
	if(precision == NBPM_FP64) return nbpm::run_peak<double>(tflops);
	if(precision == NBPM_FP32) return nbpm::run_peak<float>(tflops);
	nbpm::set_last_error("unknown precision");
	return NBPM_ERR_ARG;
}
