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
	NBPM_ERR_INTERNAL = 7,
	NBPM_ERR_TIMEOUT = 8     /* nbpm_server_wait gave up before the request finished */
};

enum { NBPM_FP64 = 0, NBPM_FP32 = 1 };

typedef struct nbpm_options {
	int precision;        /* NBPM_FP64 (default, reference parity) or NBPM_FP32 */
	int groups_per_pass;  /* wavelengths propagated together; 0 = all (batched), 1 = plain */
	int use_graph;        /* capture the slab loop in a CUDA graph (default 1) */
	int device;           /* CUDA device ordinal (default 0) */
	int verbose;          /* print the reference's progress lines to stdout */
	int tune;             /* 1 (default): the first plan of a shape times the candidate line-solve
	                         configurations and keeps the fastest (cached per shape for the
	                         process); 0: rule-based configuration, no timing runs */
	const char* solve_config; /* NULL, or "<x>;<y>" forcing one candidate per direction (as listed
	                         by nbpm_solve_candidates; either part may be "auto") */
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

/* Propagates several samples of possibly different mesh sizes in one run: every sample runs on
 * its own streams and workspace, the samples being parallel branches of one CUDA graph, so the
 * device interleaves their kernels (each sample keeps the line-solve configuration of its own
 * mesh). Results are identical to separate nbpm_run_backend_ex calls. This entry and the ones built on it (nbpm_run_backend_ex,
 * nbpm_run_backend_with/without_mask) keep the device plan of a call without bulk output and
 * reuse it when the next call has the same settings, sizes, mask formula and options: its
 * device buffers and recorded CUDA graph stay, the inputs (director, mask and its z weights)
 * are prepared and uploaded again and the results are the same. The kept plan holds its device memory until another call replaces it or
 * nbpm_release_plan_cache is called; the environment variable NBPM_PLAN_CACHE=0 turns the reuse
 * off. Concurrent calls do not share it. */
int nbpm_run_batch(int n_samples, const nbpm_sample* samples, const nbpm_options* opts,
		nbpm_timing* timing);

/* Frees the plan kept by nbpm_run_batch (no counterpart in the reference: the reference has no
 * device state between calls). Returns 0. */
int nbpm_release_plan_cache(void);

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

/* Runs the plan once without a graph, timing every kernel launch with CUDA events, each
 * kernel alone on the device (the device is synchronised before every launch, so the setup
 * and main streams do not overlap as they do in execute). Fills up to *n entries (kernel name, total ms, launches, algorithmic bytes
 * moved by those launches) and sets *n to the number of entries written. */
int nbpm_plan_profile(nbpm_plan* plan, char (*names)[48], double* ms, int* launches, double* bytes, int* n);

/* Device memory the plan holds, bytes. */
long long nbpm_plan_device_bytes(const nbpm_plan* plan);

/* Line-solve configuration of sample `sample` of the plan as "<x>;<y>" (e.g.
 * "xc:M=8:KS=4;yq:KS=2"), and in `report` (may be NULL) how it was chosen: forced, rule-based,
 * or the tuner's device time per candidate. The reference runs one sequential Thomas sweep per
 * line on every mesh (BlockSparseMatrix.cpp:195-259, 386-451); no counterpart there. */
int nbpm_plan_solve_config(const nbpm_plan* plan, int sample, char* config, int n_config, char* report,
		int n_report);

/* The candidate line-solve configurations for the mesh and slots of the JSON settings at a
 * precision and wavelengths per pass: "x=<c>|<c>...\ny=<c>|...\ndefault=<x>;<y>". Host-side
 * (uses the current device's SM count and shared memory when a device is present). No
 * counterpart in the reference. */
int nbpm_solve_candidates(const char* json_str, int precision, int groups_per_pass, char* out, int n);

/* Forgets every tuned configuration of the process (the next plan of each shape times its
 * candidates again). Returns 0. No counterpart in the reference. */
int nbpm_tune_cache_clear(void);

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
 * real-time loops that must avoid the allocator's latency and the implicit synchronisation of
 * cudaMalloc/cudaFree, and hosts that give the whole device memory to their own pool. It
 * allocates nothing: its scratch is a fixed 32 MiB device array (2 Mi complex FP64 values)
 * that every device loading the library holds until the process exits, so sizes with
 * 5*nlines*(L-1) + 2*nlines above 2*1024*1024 are rejected with NBPM_ERR_SIZE. The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress) and keeps it. The
 * call returns after the solve completed on the given stream. All calls share the array and
 * it keeps the last call's contents (every value a call reads is written earlier by the same
 * call): calls that overlap on the GPU (other streams, other host threads) race on it and must
 * be serialised by the caller. No counterpart in the reference. */
int nbpm_periodic_tridiag_solve_noalloc(int L, int nlines, const double* inf, const double* mid,
		const double* sup, const double* rhs, double* x, void* stream);

/* ---- Serving: continuous batching of samples on one GPU ----
 *
 * A thread-safe submit / poll interface over the same plans (no counterpart in the reference,
 * whose backend runs one blocking call per sample, bpm_backend.cpp:7-164). A server thread
 * admits queued requests first-come first-served while their estimated device memory fits
 * the budget, advances every request in flight by a few slabs per scheduling round
 * (each on its own CUDA streams, so requests of different meshes run side by side and new
 * ones join at slab boundaries), and copies each finished request's screen fields into its
 * E_field_vals buffer. A request runs the same launch sequence as a standalone run with the
 * same precision, so its result does not depend on the other requests. */
typedef struct nbpm_server nbpm_server;

typedef struct nbpm_server_options {
	int precision;          /* NBPM_FP32 (default) or NBPM_FP64 */
	int device;
	double hbm_budget_gb;   /* admission budget for the requests in flight (default 150) */
	int slabs_per_round;    /* slabs each request in flight advances per round when
	                           round_voxel_steps is 0 (default 8) */
	int max_active;         /* requests in flight at most; 0: limited by the budget only */
	double round_voxel_steps; /* > 0 (default 4e8): each request advances as many slabs per
	                           round as fit this many voxel-steps (at least one), so small
	                           requests finish in few rounds next to large ones */
} nbpm_server_options;

enum { NBPM_REQ_QUEUED = 0, NBPM_REQ_RUNNING = 1, NBPM_REQ_DONE = 2, NBPM_REQ_FAILED = 3, NBPM_REQ_CANCELLED = 4 };

typedef struct nbpm_request_info {
	int state;               /* NBPM_REQ_* */
	int error_code;          /* NBPM_ERR_* when FAILED */
	char error[256];
	long long voxel_steps;
	long long device_bytes;  /* admission estimate */
	double queue_ms;         /* submit -> admission */
	double latency_ms;       /* submit -> result in E_field_vals */
} nbpm_request_info;

typedef struct nbpm_server_stats {
	int queued, running;
	long long done, failed, cancelled;
	long long bytes_in_use, peak_bytes, budget_bytes;
	long long voxel_steps_done;
	int rounds;
} nbpm_server_stats;

void nbpm_default_server_options(nbpm_server_options* opts);
/* Starts the server thread; the device is first used when a request is admitted. */
int nbpm_server_create(const nbpm_server_options* opts, nbpm_server** out);
/* Cancels queued requests, lets the ones in flight finish, stops the thread. */
int nbpm_server_destroy(nbpm_server* server);
/* Validates a request (the reference's messages and codes, as nbpm_run_backend_ex) and
 * queues it; fails with NBPM_ERR_MEMORY when it alone exceeds the budget. The director, mask
 * and E_field_vals buffers are borrowed until the request is DONE, FAILED or CANCELLED. */
int nbpm_server_submit(nbpm_server* server, const nbpm_sample* request, long long* id);
int nbpm_server_poll(nbpm_server* server, long long id, nbpm_request_info* info);
/* Blocks until the request leaves the queue and the GPU (timeout_s < 0: no limit);
 * NBPM_ERR_TIMEOUT when the time runs out first. */
int nbpm_server_wait(nbpm_server* server, long long id, double timeout_s, nbpm_request_info* info);
/* Queued requests are dropped; requests in flight stop at the next round boundary. */
int nbpm_server_cancel(nbpm_server* server, long long id);
/* Forgets a finished request (its id becomes unknown). */
int nbpm_server_release(nbpm_server* server, long long id);
int nbpm_server_get_stats(nbpm_server* server, nbpm_server_stats* stats);

/* ---- Microscope stage: objective focalisation and incoherent spectra (FP64) ----
 *
 * Replaces the Python post-processing that follows the backend call:
 *   OpticalFields (HighLevelPythonInterface/nemaktis/light_propagator.py:448-719): wavevector
 *   grid :576-596, objective filter and NA mask :614-646, update_NA_objective :702-705,
 *   focus_fields :708-719;
 *   FieldViewer (nemaktis/field_viewer.py): _update_specter :348-388 and
 *   _update_averaged_specter :391-455 (Jones matrices :472-513, Koehler weights :515-518).
 * The fields stay on the device between focalisation and spectrum; the colour conversion of
 * _update_POM_image (dtmm colour tables) is not part of the library. */
typedef struct nbpm_microscope nbpm_microscope;

typedef struct nbpm_microscope_params {
	int Nx, Ny;                  /* mesh_dimensions */
	double Lx, Ly;               /* mesh_lengths (spacing L / max(1, N-1)) */
	int n_wavelengths;
	const double* wavelengths;   /* µm, n_wavelengths values */
	const double* n_out;         /* index of the output medium per wavelength; NULL: 1 */
	double max_NA_objective;
	double max_NA_condenser;
	int N_radial_wavevectors;
	int koehler_1D;
	double zfoc_NA_corr;
	int n_wavevectors;           /* > 0: explicit wavevectors (n x 2); 0: the OpticalFields grid */
	const double* wavevectors;
	int device;
} nbpm_microscope_params;

enum { NBPM_WAVEPLATE_NONE = 0, NBPM_WAVEPLATE_QUARTER = 1, NBPM_WAVEPLATE_HALF = 2, NBPM_WAVEPLATE_TINT = 3 };

/* FieldViewer optical elements (angles in degrees) and condenser aperture. */
typedef struct nbpm_viewer_settings {
	int polariser;
	double polariser_angle;
	int analyser;
	double analyser_angle;
	int lower_waveplate;         /* NBPM_WAVEPLATE_* between polariser and sample */
	double lower_waveplate_angle;
	int upper_waveplate;         /* NBPM_WAVEPLATE_* between sample and analyser */
	double upper_waveplate_angle;
	double NA_condenser;
} nbpm_viewer_settings;

/* All elements off, NA_condenser 0. */
void nbpm_default_viewer_settings(nbpm_viewer_settings* s);
/* Allocates the device buffers (two field arrays, filter tables, spectrum) and tabulates the
 * objective filter; fields start at zero. */
int nbpm_microscope_create(const nbpm_microscope_params* params, nbpm_microscope** out);
int nbpm_microscope_destroy(nbpm_microscope* m);
int nbpm_microscope_shape(const nbpm_microscope* m, int* n_wavelengths, int* n_wavevectors, int* Ny, int* Nx);
/* Wavevectors in use (n_wavevectors x 2); n must equal n_wavevectors. */
int nbpm_microscope_wavevectors(const nbpm_microscope* m, double* out, int n);
/* OpticalFields.vals setter: (Nl, Nq, 4, Ny, Nx) complex128 from host memory. */
int nbpm_microscope_set_fields(nbpm_microscope* m, const double* vals, long long n_vals);
/* The same from the device-resident output of sample `sample` of an executed plan (FP32
 * plans are widened to FP64), without a host round trip. */
int nbpm_microscope_set_fields_from_plan(nbpm_microscope* m, nbpm_plan* plan, int sample);
/* update_NA_objective(NA_objective) then focus_fields(z_focus): NA is clamped to
 * [0, max_NA_objective]. */
int nbpm_microscope_focus(nbpm_microscope* m, double z_focus, double NA_objective);
/* OpticalFields.focused_vals to host memory, (Nl, Nq, 4, Ny, Nx) complex128. */
int nbpm_microscope_get_focused(nbpm_microscope* m, double* out, long long n_vals);
/* FieldViewer._update_specter + _update_averaged_specter on the focused fields: writes the
 * q-averaged spectrum, (Ny, Nx, n_wavelengths) float64, n = Ny*Nx*n_wavelengths. */
int nbpm_microscope_spectrum(nbpm_microscope* m, const nbpm_viewer_settings* settings, double* spectrum,
		long long n);
/* Device time of the last focus and spectrum calls (ms) and device memory held (bytes). */
int nbpm_microscope_timing(const nbpm_microscope* m, double* focus_ms, double* spectrum_ms,
		long long* device_bytes);

/* Message of the last failure on this thread ("" if none). */
const char* nbpm_last_error(void);

/* Library version string. */
const char* nbpm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NBPM_H */
