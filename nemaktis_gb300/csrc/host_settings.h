// Backend settings: the subset of the reference's JSON tree read on the bpm_backend path,
// with the reference's error messages.
//
// Reference: BeamPropagationSolver/src/SettingsLib/BaseSettings.cpp:8-22 (sections),
// BaseSettings.h:59-91 (typed parse + message format), AlgorithmSettings.cpp:4-16,
// PhysicsSettings.cpp:8-83 (wavelengths :43-58, q-list :60-82), PostprocessorSettings.cpp,
// BPMIteration.cpp:21-50 (beam profile), PhysicsCoefficients.cpp:27-103 (index strings),
// PythonBackend/bpm_backend.cpp:20-31 (mesh keys, director size) and
// UtilitiesLib/VectorField.cpp:43-114 (mask and z interpolation weights).
#pragma once

#include <cmath>
#include <cstdio>
#include <regex>
#include <string>
#include <utility>
#include <vector>

#include "host_expr.h"
#include "host_json.h"

namespace nbpm {

// Error carrying the reference's message text (the reference throws std::string).
struct BackendError : std::runtime_error {
	int code;
	BackendError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

enum ErrCode { E_OK = 0, E_SETTINGS = 1, E_SIZE = 2, E_EXPR = 3, E_CUDA = 4, E_MEMORY = 5,
	E_ARG = 6, E_INTERNAL = 7 };

struct Section {
	const Json* node;
	std::string name;
	Section(const Json& parent, const std::string& n) : name(n) {
		if(parent.kind != Json::Object || !parent.has(n))
			throw BackendError(E_SETTINGS, "The section \"" + n + "\" is missing from the setting file");
		node = &parent.at(n);
	}
	[[noreturn]] void bad(const std::string& var, const std::string& what) const {
		throw BackendError(E_SETTINGS, "Error when parsing variable \"" + var + "\" in section \"" +
			name + "\":\n" + what);
	}
	const Json& get(const std::string& var) const {
		if(node->kind != Json::Object || !node->has(var)) bad(var, "key '" + var + "' not found");
		return node->at(var);
	}
	bool has(const std::string& var) const { return node->kind == Json::Object && node->has(var); }
	std::string str(const std::string& var) const {
		try { return get(var).as_string(); } catch(JsonError& e) { bad(var, e.what()); }
	}
	double num(const std::string& var) const {
		try { return get(var).as_number(); } catch(JsonError& e) { bad(var, e.what()); }
	}
	long long integer(const std::string& var) const {
		try { return get(var).as_int(); } catch(JsonError& e) { bad(var, e.what()); }
	}
	bool boolean(const std::string& var) const {
		try { return get(var).as_bool(); } catch(JsonError& e) { bad(var, e.what()); }
	}
	std::vector<double> numvec(const std::string& var) const {
		try { return get(var).as_number_array(); } catch(JsonError& e) { bad(var, e.what()); }
	}
};

struct BackendSettings {
	std::string lc_field_type, results_folder;
	int n_woodbury = 2, nz_substeps = 1;
	std::string beam_profile;
	int beam_type = 0;  // 0 UniformBeam, 1 GaussianBeam, 2 None
	double waist = 0;
	int Nx = 0, Ny = 0, Nz = 0;
	double dx = 0, dy = 0, dz = 0;
	std::string basis;
	std::string no_expr, ne_expr, ne_imag_expr, nhost_expr, nin_expr, nout_expr;
	std::vector<double> wavelengths;
	std::vector<std::pair<double, double>> q;
	bool bulk_activate = false, screen_activate = true;
	std::string bulk_base_name;
	std::vector<double> iso_thick, iso_index;
	double z_foc = 0, NA = 0;
	// Evaluated per wavelength (PhysicsCoefficients::get_*).
	std::vector<double> no, ne, ne_imag, nhost, nin, nout;
	double nout_06 = 1;
};

inline double eval_index(const std::string& e, double lambda, const char* which) {
	try {
		Expr ex(e, {"lambda"});
		return ex.eval1(lambda);
	}
	catch(ExprError&) {
		throw BackendError(E_EXPR, std::string("Wrong expression for ") + which);
	}
}

inline BackendSettings parse_settings(const std::string& json_str) {
	Json j;
	try { j = JsonReader::parse(json_str); }
	catch(JsonError& e) { throw BackendError(E_SETTINGS, std::string("[json.exception.") + e.what() + "]"); }
	const double PI_REF = 3.1415926535897932;
	BackendSettings s;
	Section alg(j, "Algorithm settings");
	Section gen(*alg.node, "General");
	s.lc_field_type = gen.str("LC field type");
	s.results_folder = gen.str("Results folder name");
	if(s.lc_field_type != "Director" && s.lc_field_type != "Q-tensor")
		throw BackendError(E_SETTINGS, "Parsing error: \"LC field type\" must be \"Director\" or \"Q-tensor\"");
	Section bpm(*alg.node, "Beam propagation");
	s.n_woodbury = (int)bpm.integer("N Woodbury steps");
	s.nz_substeps = (int)bpm.integer("Number of substeps per slab");

	Section phys(j, "Physics settings");
	Section ic(*phys.node, "Initial conditions");
	s.beam_profile = ic.str("Beam profile");
	ic.str("LC field file");
	s.basis = ic.str("Basis convention");
	if(s.basis != "XYZ" && s.basis != "YZX" && s.basis != "ZXY")
		throw BackendError(E_SETTINGS, "Parsing error: \"Basis convention\" must be \"XYZ\", \"YZX\" or \"ZXY\"");
	Section co(*phys.node, "Coefficients");
	s.no_expr = co.str("no");
	s.ne_expr = co.str("ne");
	s.ne_imag_expr = co.has("ne_imag") ? co.str("ne_imag") : "0";
	s.nhost_expr = co.has("nhost") ? co.str("nhost") : "1";
	s.nin_expr = co.has("nin") ? co.str("nin") : "1";
	s.nout_expr = co.has("nout") ? co.str("nout") : "1";
	if(co.has("Wavelengths")) s.wavelengths = co.numvec("Wavelengths");
	else {
		double mean = co.num("Mean wavelength");
		double fwhm = co.num("Spectral FWHM");
		long long n = co.integer("N wavelengths");
		if(n == 1) s.wavelengths.push_back(mean);
		else {
			s.wavelengths.resize((size_t)std::max(0LL, n));
			for(size_t i = 0; i < s.wavelengths.size(); i++)
				s.wavelengths[i] = mean + fwhm * (double(i) / (s.wavelengths.size() - 1.) - 0.5);
		}
	}
	if(co.has("Wavevectors")) {
		auto raw = co.numvec("Wavevectors");
		if(raw.size() % 2 != 0)
			throw BackendError(E_SETTINGS, "Wrong number of values for the \"Wavevectors\" entry,\nshould be a multiple of 2");
		for(size_t i = 0; i < raw.size() / 2; i++) s.q.emplace_back(raw[2 * i], raw[2 * i + 1]);
	}
	else {
		double NA = co.num("Condenser numerical aperture");
		int Nc = (int)co.integer("N radial illumination directions");
		s.q.emplace_back(0., 0.);
		for(int ir = 1; ir < Nc; ir++)
			for(int iphi = 0; iphi < 6 * ir; iphi++) {
				double phi = iphi * PI_REF / 3;
				s.q.emplace_back(ir * NA / (Nc - 1) * std::cos(phi), ir * NA / (Nc - 1) * std::sin(phi));
			}
	}

	Section post(j, "Postprocessor settings");
	Section bulk(*post.node, "Bulk output");
	s.bulk_activate = bulk.boolean("Activate");
	s.bulk_base_name = bulk.str("Base name");
	Section scr(*post.node, "Screen output");
	s.screen_activate = scr.boolean("Activate");
	scr.str("Base name");
	s.iso_thick = scr.numvec("Isotropic layer thicknesses");
	s.iso_index = scr.numvec("Isotropic layer refractive indices");
	s.z_foc = scr.num("Focalisation z-shift");
	s.NA = scr.num("Numerical aperture");

	// Mesh keys read directly by the backend entry (bpm_backend.cpp:20-26).
	try {
		auto sp = j.at("Physics settings").at("Initial conditions").at("Mesh spacings").as_number_array();
		auto dm = j.at("Physics settings").at("Initial conditions").at("Mesh dimensions").as_number_array();
		if(sp.size() < 3 || dm.size() < 3) throw JsonError("out_of_range: mesh arrays need 3 entries");
		s.dx = sp[0]; s.dy = sp[1]; s.dz = sp[2];
		s.Nx = (int)dm[0]; s.Ny = (int)dm[1]; s.Nz = (int)dm[2];
	}
	catch(JsonError& e) { throw BackendError(E_SETTINGS, std::string("[json.exception.") + e.what() + "]"); }
	if(s.Nx < 1 || s.Ny < 1 || s.Nz < 1)
		throw BackendError(E_SETTINGS, "Mesh dimensions must be positive");

	// Beam profile (BPMIteration.cpp:21-50)
	if(s.beam_profile == "UniformBeam") s.beam_type = 0;
	else if(s.beam_profile == "None") s.beam_type = 2;
	else {
		std::smatch m;
		static const std::regex re("GaussianBeam\\(([0-9]+\\.?[0-9]*)\\)");
		if(std::regex_match(s.beam_profile, m, re)) { s.beam_type = 1; s.waist = std::stod(m[1]); }
		else throw BackendError(E_SETTINGS, "Unrecognised beam profile");
	}
	if(s.iso_thick.size() != s.iso_index.size())
		throw BackendError(E_SETTINGS, "Inconsistent number of isotropic layers");

	// Index expressions, in the order the reference first evaluates them.
	for(double lam : s.wavelengths) {
		s.no.push_back(eval_index(s.no_expr, lam, "no"));
		s.ne.push_back(eval_index(s.ne_expr, lam, "ne"));
		s.ne_imag.push_back(eval_index(s.ne_imag_expr, lam, "ne_imag"));
		s.nhost.push_back(eval_index(s.nhost_expr, lam, "nhost"));
		s.nin.push_back(eval_index(s.nin_expr, lam, "nin"));
		// PhysicsCoefficients::get_nout reports its failure as "nin" (:95-101).
		s.nout.push_back(eval_index(s.nout_expr, lam, "nin"));
	}
	s.nout_06 = eval_index(s.nout_expr, 0.6, "nin");
	return s;
}

// Mask values and per-cell interpolation weights (VectorField.cpp:43-114). mask_out gets
// (val >= 0) per voxel; w_out gets 2 weights per voxel of the first Nz-1 planes. If the
// formula's sign changes disagree with the mask, the reference prints a notice and falls
// back to 0.5/0.5 everywhere (its resize at :111 truncates the array; the evident intent,
// uniform weights, is applied here).
inline void mask_weights(const BackendSettings& s, const double* mask_vals, const std::string& formula,
		std::vector<unsigned char>& mask_out, std::vector<double>& w_out) {
	int Nx = s.Nx, Ny = s.Ny, Nz = s.Nz;
	size_t nv = (size_t)Nx * Ny * Nz;
	mask_out.resize(nv);
	#pragma omp parallel for schedule(static)
	for(long long i = 0; i < (long long)nv; i++) mask_out[i] = mask_vals[i] >= 0;
	const size_t nw = 2 * (size_t)Nx * Ny * (Nz > 1 ? Nz - 1 : 0);
	w_out.resize(nw);
	#pragma omp parallel for schedule(static)
	for(long long i = 0; i < (long long)nw; i++) w_out[i] = 0.5;
	if(formula.empty() || Nz < 2) return;
	Expr ex;
	try { ex = Expr(formula, {"x", "y", "z"}); }
	catch(ExprError& e) { throw BackendError(E_EXPR, std::string("Wrong mask formula: ") + e.what()); }
	int failed = 0;
	#pragma omp parallel for reduction(|:failed) schedule(dynamic, 64)
	for(long long iperp = 0; iperp < (long long)Nx * Ny; iperp++) {
		int ix = (int)(iperp % Nx), iy = (int)(iperp / Nx);
		double v[3] = {(ix - 0.5 * (Nx - 1)) * s.dx, (iy - 0.5 * (Ny - 1)) * s.dy, 0};
		// the formula at the upper plane of a cell is the one at the lower plane of the next
		// (the same z), so each plane is evaluated once
		double f_next = 0;
		for(int iz = 0; iz < Nz - 1; iz++) {
			size_t i = iperp + (size_t)Nx * Ny * iz;
			double zi = (iz - 0.5 * (Nz - 1)) * s.dz, zm = zi, zp = (iz + 1 - 0.5 * (Nz - 1)) * s.dz;
			double& z = v[2];
			double fm;
			if(iz == 0) { z = zm; fm = ex.eval(v); }
			else fm = f_next;
			z = zp; double fp = ex.eval(v);
			f_next = fp;
			if(fm * fp <= 0) {
				if(mask_out[i] == mask_out[i + (size_t)Nx * Ny]) failed = 1;
				// bisection to 1e-3 dz; fm always holds the formula at zm
				while(std::abs(zp - zm) >= 1e-3 * s.dz) {
					z = 0.5 * (zp + zm); double f = ex.eval(v);
					if(f == 0) break;
					else if(f * fm < 0) zp = z;
					else { zm = z; fm = f; }
				}
				w_out[2 * i] = (z - zi) / s.dz;
				w_out[2 * i + 1] = 1 - w_out[2 * i];
			}
		}
	}
	if(failed) {
		std::printf("Mask values do not corresponds to the given formula, will ignore interpolation correction\n");
		std::fill(w_out.begin(), w_out.end(), 0.5);
	}
}

}  // namespace nbpm
