// Line-solve configurations of one sample: the kernel family and its chunking / slots-per-thread
// for the x-lines and for the y-lines, the candidates a plan may run for a mesh, the rule-based
// default, and the text form used by the tuner's cache and by nbpm_options.solve_config.
//
// The reference solves every line with one sequential Thomas sweep per OpenMP thread
// (BlockSparseMatrix.cpp:195-259, 386-451) whatever the mesh; here the best mapping of lines to
// threads depends on the mesh and the number of (q, pol) slots per wavelength, so the plan times
// the candidates once per shape (nbpm.cu, Plan::tune) and keeps the fastest.
#pragma once

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

namespace nbpm {

// (M, KS) pairs with compiled chunked-kernel instances (k_solve_xc / k_solve_yc).
inline bool solve_pair_ok(int M, int KS) {
	switch(M) {
		case 2: case 4: case 8: return KS == 1 || KS == 2 || KS == 4;
		case 16: return KS == 1 || KS == 2;
		case 32: return KS == 1;
	}
	return false;
}

struct SolveCfg {
	// x-lines: Mx == 0 sequential (k_stencil + k_solve); WPLx > 1 several warps per line
	// (k_solve_xw, 8-point chunks); xs chunk values in shared memory (k_solve_xs); else one warp
	// per line with M-point lane chunks (k_solve_xc). KSx slots per thread.
	int Mx = 0, KSx = 1, WPLx = 1;
	bool xs = false;
	// y-lines: yq > 0 sequential per column (k_solve_yq, yq slots per thread); ys chunks held in
	// a scratch field (k_solve_ys, KSy slots); My > 0 32 columns x WY warps of M-row chunks
	// (k_solve_yc, KSy slots; y1024w: the Woodbury solves with 32 warps of 8-row chunks and 2
	// slots per thread); else sequential (k_stencil + k_solve).
	// Mt > 0: one warp per column with Mt-row lane chunks (k_solve_yt, KSy slots). Mxt > 0: the
	// y-lines solved as x-lines of the transposed frame (k_solve_xc on transposed fields and
	// coefficients, Mxt-point lane chunks, KSy slots); needs the x-lines on k_solve_xc, whose last
	// Woodbury solve hands the fields over transposed, and two Woodbury steps.
	// WPLt > 1: the transposed frame's x-lines on k_solve_xw (WPLt warps per line, Mxt = 8).
	int My = 0, WY = 0, KSy = 1, yq = 0, Mt = 0, Mxt = 0, WPLt = 1;
	bool ys = false, y1024w = false;
	// factor plane sizes (elements per factor and line set), from the x layout
	size_t plane_x = 0, plane_y = 0;

	std::string xstr() const {
		char b[64];
		if(Mx == 0) return "xseq";
		if(WPLx > 1) std::snprintf(b, sizeof b, "xw:M=%d:KS=%d:W=%d", Mx, KSx, WPLx);
		else if(xs) std::snprintf(b, sizeof b, "xs:M=%d:KS=%d", Mx, KSx);
		else std::snprintf(b, sizeof b, "xc:M=%d:KS=%d", Mx, KSx);
		return b;
	}
	std::string ystr() const {
		char b[64];
		if(yq) std::snprintf(b, sizeof b, "yq:KS=%d", yq);
		else if(Mt) std::snprintf(b, sizeof b, "yt:M=%d:KS=%d", Mt, KSy);
		else if(Mxt && WPLt > 1) std::snprintf(b, sizeof b, "yx:M=%d:KS=%d:W=%d", Mxt, KSy, WPLt);
		else if(Mxt) std::snprintf(b, sizeof b, "yx:M=%d:KS=%d", Mxt, KSy);
		else if(ys) std::snprintf(b, sizeof b, "ys:KS=%d", KSy);
		else if(My) std::snprintf(b, sizeof b, "yc:M=%d:KS=%d:W=%d%s", My, KSy, WY, y1024w ? ":W1024" : "");
		else return "yseq";
		return b;
	}
	std::string str() const { return xstr() + ";" + ystr(); }
	void set_x(const SolveCfg& o) { Mx = o.Mx; KSx = o.KSx; WPLx = o.WPLx; xs = o.xs; }
	void set_y(const SolveCfg& o) {
		My = o.My; WY = o.WY; KSy = o.KSy; yq = o.yq; Mt = o.Mt; Mxt = o.Mxt; WPLt = o.WPLt; ys = o.ys;
		y1024w = o.y1024w;
	}
	// x on k_solve_xc or k_solve_xw: the kernels whose last Woodbury solve can hand the fields over
	// to the transposed frame
	bool x_hands_over() const { return Mx > 0 && !xs; }
};

// What the choice depends on.
struct SolveShape {
	int Nx = 0, Ny = 0;
	int spg = 2;        // slots (q, pol) per wavelength
	int ng = 1;         // wavelengths per pass
	int nw = 2;         // Woodbury steps
	bool fp32 = false;
	int nsm = 152;      // streaming multiprocessors
	size_t smem = 227 * 1024;  // opt-in shared memory per block
	bool relax = false;  // every compiled instance (forced configurations), not only the timed set
	size_t csize() const { return fp32 ? 8 : 16; }
	// chunk values (M * KS complex) kept per thread
	int cap() const { return fp32 || relax ? 32 : 16; }
};

inline size_t plane_x_of(const SolveCfg& c, const SolveShape& s) {
	size_t N = (size_t)s.Nx * s.Ny;
	return c.Mx ? std::max(N, (size_t)s.Ny * 32 * c.WPLx * c.Mx) : N;
}

inline void finalize(SolveCfg& c, const SolveShape& s) {
	c.plane_x = plane_x_of(c, s);
	// transposed-frame y factors: the chunk-interleaved x layout of Nx lines of 32 * Mxt points
	c.plane_y = std::max((size_t)s.Nx * s.Ny, c.Mxt ? (size_t)s.Nx * 32 * c.WPLt * c.Mxt : (size_t)0);
}

inline bool xs_fits(int ks, int M, const SolveShape& s) { return (size_t)4 * ks * 32 * (M + 1) * s.csize() <= 100 * 1024; }
inline bool xw_fits(int ks, int wpl, const SolveShape& s) {
	return ((size_t)ks * 32 * wpl * 9 + 4 * ks * wpl + 2 * ks) * s.csize() <= s.smem;
}
inline bool yc_fits(int M, int ks, int WY, const SolveShape& s) {
	return ((size_t)(4 + 3 * ks) * WY * 32 + (size_t)ks * 32) * s.csize() <= s.smem;
}

// Candidates for the x-lines (y fields left at their defaults). relaxed: every configuration
// with a compiled instance (chunk values up to 32 complex per thread in either precision), the
// set a forced configuration is checked against; the tuner times the default set.
inline std::vector<SolveCfg> x_candidates(const SolveShape& s0, bool relaxed = false) {
	SolveShape s = s0;
	if(relaxed) s.relax = true;
	std::vector<SolveCfg> out;
	const int ux = s.Nx - 1;
	if(s.Nx > 3) {
		if(ux <= 1024) {
			int M0 = 0;
			for(int M = 2; M <= 32; M *= 2) if(32 * M >= ux) { M0 = M; break; }
			for(int ks : {4, 2, 1})
				if(s.spg % ks == 0 && solve_pair_ok(M0, ks) && (M0 * ks <= s.cap() || ks == 1)) {
					SolveCfg c; c.Mx = M0; c.KSx = ks; out.push_back(c);
				}
			if(M0 == 32)
				for(int ks : {4, 2, 1})
					if(s.spg % ks == 0 && xs_fits(ks, 32, s)) { SolveCfg c; c.Mx = 32; c.KSx = ks; c.xs = true; out.push_back(c); }
		}
		if(ux > 256 && ux <= 2048) {
			const int wpl = (ux + 255) / 256;
			for(int ks : {4, 2, 1})
				if(s.spg % ks == 0 && (8 * ks <= s.cap() || ks == 1) && xw_fits(ks, wpl, s)) {
					SolveCfg c; c.Mx = 8; c.KSx = ks; c.WPLx = wpl; out.push_back(c);
				}
		}
	}
	if(out.empty()) out.push_back(SolveCfg());
	for(auto& c : out) finalize(c, s);
	return out;
}

// Candidates for the y-lines (x fields left at their defaults); relaxed as for x_candidates.
inline std::vector<SolveCfg> y_candidates(const SolveShape& s0, bool relaxed = false) {
	SolveShape s = s0;
	if(relaxed) s.relax = true;
	std::vector<SolveCfg> out;
	const int uy = s.Ny - 1;
	if(s.Ny > 3) {
		int M0 = 0;
		for(int M = 2; M <= 32; M *= 2) if((uy + M - 1) / M <= 16) { M0 = M; break; }
		if(M0) {
			const int WY = (uy + M0 - 1) / M0;
			for(int ks : {4, 2, 1})
				if(s.spg % ks == 0 && solve_pair_ok(M0, ks) && (M0 * ks <= s.cap() || ks == 1) && yc_fits(M0, ks, WY, s)) {
					SolveCfg c; c.My = M0; c.WY = WY; c.KSy = ks; out.push_back(c);
					if(uy > 128 && uy <= 256 && s.spg % 2 == 0 && ks >= 2) { c.y1024w = true; out.push_back(c); }
				}
		}
		if(uy <= 1024) {
			int Mt = 0;
			for(int M = 2; M <= 32; M *= 2) if(32 * M >= uy) { Mt = M; break; }
			for(int ks : {4, 2, 1})
				if(s.spg % ks == 0 && solve_pair_ok(Mt, ks) && (Mt * ks <= s.cap() || ks == 1)) {
					SolveCfg c; c.Mt = Mt; c.KSy = ks; out.push_back(c);
					if(s.Nx > 3 && s.nw == 2) { SolveCfg t; t.Mxt = Mt; t.KSy = ks; out.push_back(t); }
				}
		}
		// long y-lines as several-warps-per-line x-lines of the transposed frame
		if(uy > 256 && uy <= 2048 && s.Nx > 3 && s.nw == 2) {
			const int wpl = (uy + 255) / 256;
			for(int ks : {4, 2, 1})
				if(s.spg % ks == 0 && (8 * ks <= s.cap() || ks == 1) && xw_fits(ks, wpl, s)) {
					SolveCfg t; t.Mxt = 8; t.WPLt = wpl; t.KSy = ks; out.push_back(t);
				}
		}
		for(int ks : {4, 2, 1})
			if(s.spg % ks == 0) { SolveCfg c; c.yq = ks; out.push_back(c); }
		for(int ks : {2, 1})
			if(s.spg % ks == 0) { SolveCfg c; c.ys = true; c.KSy = ks; out.push_back(c); }
		if(!M0) out.push_back(SolveCfg());
	}
	if(out.empty()) out.push_back(SolveCfg());
	for(auto& c : out) finalize(c, s);
	return out;
}

// Rule-based default (the configuration used without tuning).
inline SolveCfg heuristic(const SolveShape& s) {
	SolveCfg sc;
	const int ux = s.Nx - 1, uy = s.Ny - 1;
	if(s.Nx > 3) {
		for(int M = 2; M <= 32; M *= 2) if(32 * M >= ux) { sc.Mx = M; break; }
		if(ux > 256 && ux <= 2048) { sc.Mx = 8; sc.WPLx = (ux + 255) / 256; }
	}
	if(s.Ny > 3) {
		for(int M = 2; M <= 32; M *= 2) if((uy + M - 1) / M <= 16) { sc.My = M; break; }
		if(sc.My) sc.WY = (uy + sc.My - 1) / sc.My;
		if(s.fp32 && uy > 128 && uy <= 256 && s.spg % 2 == 0) sc.y1024w = true;
	}
	auto pick_ks = [&](int M) {
		for(int ks : {4, 2, 1})
			if(s.spg % ks == 0 && solve_pair_ok(M, ks) && (M * ks <= s.cap() || ks == 1)) return ks;
		return 0;
	};
	if(sc.Mx) { sc.KSx = pick_ks(sc.Mx); if(!sc.KSx) { sc.Mx = 0; sc.WPLx = 1; sc.KSx = 1; } }
	if(sc.My) { sc.KSy = pick_ks(sc.My); if(!sc.KSy) { sc.My = 0; sc.WY = 0; sc.y1024w = false; sc.KSy = 1; } }
	// small grids leave SMs idle: fewer slots per thread, more blocks
	const size_t want = 2 * (size_t)s.nsm;
	auto xblocks = [&](int ks) { return (size_t)((s.Ny + 3) / 4) * 2 * s.ng * (s.spg / ks); };
	auto yblocks = [&](int ks) { return (size_t)((s.Nx + 31) / 32) * 2 * s.ng * (s.spg / ks); };
	if(sc.Mx && sc.WPLx == 1)
		while(sc.KSx > 1 && xblocks(sc.KSx) < want && solve_pair_ok(sc.Mx, sc.KSx / 2)) sc.KSx /= 2;
	if(sc.My)
		while(sc.KSy > 1 && yblocks(sc.KSy) < want && solve_pair_ok(sc.My, sc.KSy / 2)) sc.KSy /= 2;
	if(sc.KSy < 2) sc.y1024w = false;
	// FP64 (bound by the FP64 pipe) with short y-lines on few blocks: chunks in a scratch field
	// with one slot per thread, measured 2x faster on GB300 for 64x64 meshes
	if(!s.fp32 && sc.My && sc.My <= 4 && yblocks(1) < (size_t)s.nsm) { sc.My = 0; sc.WY = 0; sc.ys = true; sc.KSy = 1; }
	if(sc.WPLx == 1 && sc.Mx >= 32) {
		sc.xs = true;
		sc.KSx = 1;
		for(int ks : {4, 2}) if(s.spg % ks == 0 && xs_fits(ks, sc.Mx, s)) { sc.KSx = ks; break; }
	}
	if(sc.My && !yc_fits(sc.My, sc.KSy, sc.WY, s)) { sc.My = 0; sc.WY = 0; sc.KSy = 1; sc.y1024w = false; }
	finalize(sc, s);
	return sc;
}

}  // namespace nbpm
