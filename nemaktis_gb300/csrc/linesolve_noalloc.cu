// Allocation-free variant of the periodic tridiagonal line solve.
//
// nbpm_periodic_tridiag_solve allocates its factorisation scratch on each call. Some callers
// cannot do that: real-time loops that must not pay the allocator's latency or the implicit
// device synchronisation of cudaMalloc/cudaFree, and hosts that hand the whole device memory
// to their own pool and forbid any other allocation. This entry point takes its scratch from a
// fixed array in device memory that the library reserves when it is loaded, so a call
// allocates nothing; the caller still provides the inputs and the output. The call is
// synchronous: it returns after the solve has completed on the given stream.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/nbpm.h"
#include "cplx.cuh"

namespace nbpm {

void set_last_error(const std::string& m);
size_t pt_scratch_elems(int L, int nlines);
int pt_check(int L, int nlines, const void* a, const void* b, const void* c, const void* d, const void* e,
	std::string& err);
int pt_run(int L, int nlines, const double* inf, const double* mid, const double* sup, const double* rhs,
	double* x, cudaStream_t st, cx<double>* scr, std::string& err);

// Fixed scratch: 2 Mi complex FP64 values (32 MiB) per device that loads the library, held
// until the process exits.
constexpr size_t NOALLOC_SCRATCH_ELEMS = (size_t)2 << 20;
static __device__ __align__(256) cx<double> g_noalloc_scratch[NOALLOC_SCRATCH_ELEMS];

// Device address of the scratch array, looked up once per device (with that device current)
// and kept. In host code the symbol g_noalloc_scratch is only a host-side stand-in, never a
// device address. A kept address is checked against the runtime before use: after a
// cudaDeviceReset the module is loaded again and the address is looked up anew.
static std::mutex g_noalloc_mu;
static cx<double>* g_noalloc_addr[256] = {};

static bool noalloc_addr_valid(cx<double>* p, int dev) {
	cudaPointerAttributes a;
	if(cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
	return a.type == cudaMemoryTypeDevice && a.device == dev && a.devicePointer == static_cast<void*>(p);
}

static cx<double>* noalloc_scratch(std::string& err) {
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if(e != cudaSuccess) { err = cudaGetErrorString(e); return nullptr; }
	if(dev < 0 || dev >= 256) { err = "device ordinal out of range"; return nullptr; }
	std::lock_guard<std::mutex> lk(g_noalloc_mu);
	if(!g_noalloc_addr[dev] || !noalloc_addr_valid(g_noalloc_addr[dev], dev)) {
		void* p = nullptr;
		e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if(e != cudaSuccess || !p) {
			err = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
			return nullptr;
		}
		g_noalloc_addr[dev] = static_cast<cx<double>*>(p);
	}
	return g_noalloc_addr[dev];
}

}  // namespace nbpm

using namespace nbpm;

extern "C" {

int nbpm_periodic_tridiag_solve_noalloc(int L, int nlines, const double* inf, const double* mid,
		const double* sup, const double* rhs, double* x, void* stream) {
	std::string err;
	int rc = pt_check(L, nlines, inf, mid, sup, rhs, x, err);
	if(rc) { set_last_error(err); return rc; }
	size_t need = pt_scratch_elems(L, nlines);
	if(need > NOALLOC_SCRATCH_ELEMS) {
		char msg[256];
		std::snprintf(msg, sizeof msg,
			"nbpm_periodic_tridiag_solve_noalloc: L=%d, nlines=%d need %zu scratch values, above the fixed "
			"maximum of %zu (5*nlines*(L-1) + 2*nlines <= %zu); use nbpm_periodic_tridiag_solve",
			L, nlines, need, NOALLOC_SCRATCH_ELEMS, NOALLOC_SCRATCH_ELEMS);
		set_last_error(msg);
		return NBPM_ERR_SIZE;
	}
	cx<double>* scr = noalloc_scratch(err);
	if(!scr) { set_last_error(err); return NBPM_ERR_CUDA; }
	cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
	// Every scratch value the kernels read is written earlier in the same call, so nothing
	// needs clearing between calls.
	rc = pt_run(L, nlines, inf, mid, sup, rhs, x, st, scr, err);
	if(rc) { set_last_error(err); return rc; }
	cudaError_t e = cudaStreamSynchronize(st);
	if(e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return NBPM_ERR_CUDA; }
	return 0;
}

}  // extern "C"
