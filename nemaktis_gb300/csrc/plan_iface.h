// Internal interface of a propagation plan, shared by the C-ABI entry points, the serving
// loop and the stages that consume a plan's device-resident output (objective focalisation,
// spectra) without a round trip through the host.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <memory>
#include <string>
#include <vector>

#include "../../include/nbpm.h"

namespace nbpm {

struct PlanFieldsView {
	const void* ptr = nullptr;  // (Nl, Nq, 4, Ny, Nx) complex, FP64 or FP32 (fp32 != 0)
	size_t n = 0;               // complex values
	int fp32 = 0;
	int Nx = 0, Ny = 0, Nl = 0, Nq = 0;
	int device = 0;
	cudaStream_t stream = nullptr;  // the plan's stream; the fields are final once it is idle
};

struct PlanBase {
	virtual ~PlanBase() {}
	virtual void upload() = 0;
	virtual void execute(nbpm_timing* t) = 0;
	virtual void download() = 0;
	// Host-side outputs once the run has finished (bulk-output files); download() calls it.
	virtual void host_finish() = 0;
	// Whether the plan may be kept for a later call with the same settings (no bulk output), and
	// pointing a kept plan at a new call's host arrays (false: the call needs a new plan).
	virtual bool reusable() const = 0;
	virtual bool rebind(int n_samples, const nbpm_sample* samples) = 0;
	virtual bool fields_view(int sample, PlanFieldsView& v) const = 0;
	// Resumable execution of a one-sample plan with every wavelength in one pass (serving):
	// step_begin records the entrance, step_advance up to n more slabs (returns the slabs
	// left), step_finish the exit, screen filter and the copy to the user buffer. All launches
	// are asynchronous on the plan's streams; step_done polls for the end of that copy.
	virtual void step_begin() = 0;
	virtual int step_advance(int nslabs) = 0;
	virtual void step_finish() = 0;
	virtual bool step_done() = 0;
	// Waits for every launch issued so far on the plan's streams.
	virtual void sync() = 0;
	// Device memory the plan will hold, from the host-side settings alone (before setup_device).
	virtual long long estimate_bytes() = 0;
	// Streams, events, buffers; the first call that touches the device.
	virtual void setup_device() = 0;
	virtual long long voxel_steps() const = 0;
	// Slabs of a one-sample plan (Nz - 1).
	virtual int slabs() const = 0;
	virtual long long device_bytes() const = 0;
	virtual double slab_ms() const = 0;
	virtual void profile(std::vector<std::string>& names, std::vector<double>& ms, std::vector<int>& cnt,
		std::vector<double>& bytes) = 0;
	// Line-solve configuration of a sample ("<x>;<y>", solve_config.h) and how it was chosen
	// (forced, rule-based, or the tuner's timings); false for an index out of range.
	virtual bool solve_config(int sample, std::string& cfg, std::string& note) const = 0;
};

// Parses and validates the samples (host only; throws BackendError); the device is not
// touched until setup_device().
std::unique_ptr<PlanBase> make_plan_host(int n_samples, const nbpm_sample* samples, const nbpm_options& opts);

// Fills v for sample `sample` of the plan; false for an index out of range.
bool plan_fields_view(nbpm_plan* p, int sample, PlanFieldsView& v);

void set_last_error(const std::string& m);

}  // namespace nbpm
