// Bench-only probe (not part of libnbpm): FMA throughput of the GPU in FP32 and FP64, the
// compute ceilings the benchmark reports beside the HBM roofline. Each thread runs independent
// FMA chains in registers; the result is written so the compiler keeps the work. Built into
// its own library (nemaktis_gb300/_build/libnbpm_bench.so) by nemaktis_gb300/build.py.
#include <cuda_runtime.h>

namespace nbpm_bench {

static const char* g_err = "";
static void set_last_error(const char* m) { g_err = m; }

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
	if(e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return 4; }
	double flops = 2.0 * (double)blocks * threads * iters * CH;
	*tflops = flops / (ms * 1e-3) / 1e12;
	return 0;
}

}  // namespace nbpm_bench

// precision: 0 = FP64, 1 = FP32. Returns 0, or 4 (CUDA error) / 6 (bad argument).
extern "C" int nbpm_bench_fma_peak(int precision, double* tflops) {
	if(!tflops) { nbpm_bench::set_last_error("null argument"); return 6; }
	if(precision == 0) return nbpm_bench::run_peak<double>(tflops);
	if(precision == 1) return nbpm_bench::run_peak<float>(tflops);
	nbpm_bench::set_last_error("unknown precision");
	return 6;
}

extern "C" const char* nbpm_bench_last_error(void) { return nbpm_bench::g_err; }
