/*
 * nbpm — GB300-native (sm_103a) beam-propagation backend for Nemaktis.
 *
 * C ABI of libnbpm.so. Plain pointers and sizes only; complex arrays are interleaved
 * (re, im) float64 pairs and their sizes count complex values, as in the reference.
 * Every entry point returns 0 on success or a non-zero NBPM_ERR_* code; the message of the
 * last failure on the calling thread is available from nbpm_last_error().
 */
#ifndef NBPM_H
#define NBPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
	NBPM_OK = 0,
	NBPM_ERR_SETTINGS = 1,  /* malformed or incomplete JSON settings */
	NBPM_ERR_SIZE = 2,      /* array sizes inconsistent with the settings */
	NBPM_ERR_EXPR = 3,      /* refractive-index or mask expression cannot be evaluated */
	NBPM_ERR_CUDA = 4,      /* CUDA runtime failure (no device, launch error, ...) */
	NBPM_ERR_MEMORY = 5,    /* device memory exhausted or above the configured budget */
	NBPM_ERR_ARG = 6,       /* invalid argument (null pointer, bad option, bad handle) */
	NBPM_ERR_INTERNAL = 7
};

enum { NBPM_FP64 = 0, NBPM_FP32 = 1 };

typedef struct nbpm_options {
	int precision;        /* NBPM_FP64 (default, reference parity) or NBPM_FP32 */
	int groups_per_pass;  /* wavelengths propagated together; 0 = all (batched), 1 = plain */
	int use_graph;        /* capture the slab loop in a CUDA graph (default 1) */
	int device;           /* CUDA device ordinal (default 0) */
	int verbose;          /* print the reference's progress lines to stdout */
} nbpm_options;

typedef struct nbpm_timing {
	double upload_ms;     /* host -> device copies */
	double compute_ms;    /* propagation + screen filter on the device */
	double download_ms;   /* device -> host copies */
	double total_ms;
	long long voxel_steps;
	int kernel_launches;  /* kernels launched by the last compute */
} nbpm_timing;

/* Fills *opts with the defaults (FP64, all wavelengths per pass, graphs on, device 0). */
void nbpm_default_options(nbpm_options* opts);

/* Replaces run_backend_without_mask, BeamPropagationSolver/src/PythonBackend/bpm_backend.h:4-7
 * (bpm_backend.cpp:7-83): JSON settings, director or Q-tensor values (Nz,Ny,Nx,3|6) float64,
 * fields (Nl,Nq,4,Ny,Nx) complex128 read (Beam profile "None") and written in place.
 * Runs with the default options (FP64). */
int nbpm_run_backend_without_mask(const char* json_str, const double* lc_field_vals, int n_lc_vals,
		double* E_field_vals, int n_E_vals);

/* Replaces run_backend_with_mask, bpm_backend.h:9-13 (bpm_backend.cpp:85-164): as above plus
 * a mask (Nz,Ny,Nx) float64 (inside <=> value >= 0) and an optional mask formula in x, y, z
 * used for the z interpolation weights. */
int nbpm_run_backend_with_mask(const char* json_str, const char* mask_formula,
		const double* lc_field_vals, int n_lc_vals, const double* mask_vals, int n_mask_vals,
		double* E_field_vals, int n_E_vals);

/* Either entry point with explicit options (mask_vals == NULL: no mask). Also fills *timing
 * when it is non-NULL. No counterpart in the reference beyond the two calls above. */
int nbpm_run_backend_ex(const char* json_str, const char* mask_formula,
		const double* lc_field_vals, int n_lc_vals, const double* mask_vals, int n_mask_vals,
		double* E_field_vals, int n_E_vals, const nbpm_options* opts, nbpm_timing* timing);

/* One sample of a batched run: the arguments of nbpm_run_backend_ex for one sample. */
typedef struct nbpm_sample {
	const char* json_str;
	const char* mask_formula;   /* may be NULL */
	const double* lc_field_vals;
	int n_lc_vals;
	const double* mask_vals;    /* may be NULL */
	int n_mask_vals;
	double* E_field_vals;
	int n_E_vals;
} nbpm_sample;

/* Propagates several samples of possibly different mesh sizes in one run (each slab step
 * advances every sample that still has slabs left). Results are identical to separate
 * nbpm_run_backend_ex calls. */
int nbpm_run_batch(int n_samples, const nbpm_sample* samples, const nbpm_options* opts,
		nbpm_timing* timing);

/* Device-resident plan: inputs are validated and uploaded once, nbpm_plan_execute runs the
 * propagation + screen filter on the device only (no host copies), nbpm_plan_download copies
 * the fields to the E_field_vals buffers given at creation. */
typedef struct nbpm_plan nbpm_plan;
int nbpm_plan_create(int n_samples, const nbpm_sample* samples, const nbpm_options* opts,
		nbpm_plan** out);
int nbpm_plan_upload(nbpm_plan* plan);
int nbpm_plan_execute(nbpm_plan* plan, nbpm_timing* timing);
int nbpm_plan_download(nbpm_plan* plan);
/* Propagation-only timing of the last execute (ms), for roofline reports: time of the slab
 * loop kernels, excluding setup and screen filter. */
int nbpm_plan_slab_ms(nbpm_plan* plan, double* ms);
int nbpm_plan_destroy(nbpm_plan* plan);

/* Runs the plan once without a graph, timing every kernel launch with CUDA events on the
 * plan's stream. Fills up to *n entries (kernel name, total ms, launches, algorithmic bytes
 * moved by those launches) and sets *n to the number of entries written. */
int nbpm_plan_profile(nbpm_plan* plan, char (*names)[48], double* ms, int* launches, double* bytes, int* n);

/* Device memory the plan holds, bytes. */
long long nbpm_plan_device_bytes(const nbpm_plan* plan);

/* Evaluates a refractive-index expression in the variable "lambda" (µm) with the backend's
 * expression evaluator (the reference uses muParser, PhysicsCoefficients.cpp:27-103). */
int nbpm_eval_index(const char* expr, double lambda, double* out);

/* Mask (value >= 0) and z interpolation weights (2 per voxel of the first Nz-1 planes) as the
 * backend computes them from a mask array and formula (VectorField.cpp:43-114). mask_out holds
 * Nx*Ny*Nz bytes, weights_out 2*Nx*Ny*(Nz-1) doubles. */
int nbpm_mask_weights(const char* json_str, const char* mask_formula, const double* mask_vals, int n_mask_vals,
		unsigned char* mask_out, double* weights_out);

/* Batched periodic tridiagonal solves on the device, complex FP64 (interleaved re, im).
 * Replaces BlockSparseMatrixDX/DY::shifted_block_vmult_inv (BeamPropagationSolver/src/
 * BeamPropagationLib/BlockSparseMatrix.cpp:195-258, 386-449) as a standalone primitive: each
 * of the nlines lines has L points, the last duplicating the first (period L-1), and row i
 * reads inf[i]*x[i-1] + mid[i]*x[i] + sup[i]*x[i+1] = rhs[i] with indices modulo L-1.
 * inf, mid, sup, rhs and x are device arrays of nlines*L complex values (line-major; entry
 * L-1 of inf/mid/sup/rhs is ignored, x[L-1] receives x[0]). Requires L >= 4. stream is a
 * cudaStream_t (NULL: default stream); the call returns after the solve completed. Allocates
 * its factorisation scratch (5*nlines*(L-1) + 2*nlines complex) stream-ordered. */
int nbpm_periodic_tridiag_solve(int L, int nlines, const double* inf, const double* mid, const double* sup,
		const double* rhs, double* x, void* stream);

/* Same solve as nbpm_periodic_tridiag_solve for callers that cannot allocate device memory:
 * code recording inside a CUDA stream capture (a cudaMalloc there breaks the capture),
 * real-time loops that must avoid the allocator and its implicit synchronisation, and hosts
 * that give the whole device memory to their own pool. It allocates nothing: its scratch is a
 * fixed 32 MiB device array (2 Mi complex FP64 values) that every device loading the library
 * holds until the process exits, so sizes with 5*nlines*(L-1) + 2*nlines above 2*1024*1024
 * are rejected with NBPM_ERR_SIZE. The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress); make that first call before any stream capture. All calls
 * share the array: calls that overlap on the GPU (other streams, other host threads) race on
 * it and must be serialised by the caller. No counterpart in the reference. */
int nbpm_periodic_tridiag_solve_noalloc(int L, int nlines, const double* inf, const double* mid,
		const double* sup, const double* rhs, double* x, void* stream);

/* Message of the last failure on this thread ("" if none). */
const char* nbpm_last_error(void);

/* Library version string. */
const char* nbpm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NBPM_H */
