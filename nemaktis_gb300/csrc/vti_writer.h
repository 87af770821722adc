// Writer of the bulk-output file: VTK XML ImageData (.vti), raw appended data, the arrays of
// BulkOpticalFieldCollection (BeamPropagationSolver/src/BeamLib/OpticalFieldCollection.cpp:
// 75-148): field data "lambda", "qx", "qy"; for each (wavelength, q, input polarisation) the
// point arrays E_real_inputX_<q>_<lambda> / E_imag_... (and inputY), three components
// (Ex, Ey, 0) per mesh point, x fastest; origin at the mesh centre. Written without VTK.
#pragma once

#include <sys/stat.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace nbpm {

struct VtiArray {
	std::string name;
	int ncomp;
	const double* data;
	size_t ntuples;
};

// Returns an empty string on success, else the reason.
inline std::string write_vti(const std::string& path, int Nx, int Ny, int Nz, double dx, double dy, double dz,
		const std::vector<VtiArray>& field_data, const std::vector<VtiArray>& point_data) {
	FILE* f = std::fopen(path.c_str(), "wb");
	if(!f) return "cannot open " + path + " for writing";
	std::string x;
	char buf[512];
	x += "<?xml version=\"1.0\"?>\n";
	x += "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n";
	std::snprintf(buf, sizeof buf,
		"  <ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"%.17g %.17g %.17g\" Spacing=\"%.17g %.17g %.17g\" "
		"Direction=\"1 0 0 0 1 0 0 0 1\">\n", Nx - 1, Ny - 1, Nz - 1, -dx * (Nx - 1) / 2., -dy * (Ny - 1) / 2.,
		-dz * (Nz - 1) / 2., dx, dy, dz);
	x += buf;
	uint64_t offset = 0;
	auto decl = [&](const VtiArray& a, const char* indent) {
		std::snprintf(buf, sizeof buf,
			"%s<DataArray type=\"Float64\" Name=\"%s\" NumberOfComponents=\"%d\" NumberOfTuples=\"%zu\" "
			"format=\"appended\" offset=\"%llu\"/>\n", indent, a.name.c_str(), a.ncomp, a.ntuples,
			(unsigned long long)offset);
		x += buf;
		offset += sizeof(uint64_t) + (uint64_t)a.ncomp * a.ntuples * sizeof(double);
	};
	x += "    <FieldData>\n";
	for(auto& a : field_data) decl(a, "      ");
	x += "    </FieldData>\n";
	std::snprintf(buf, sizeof buf, "    <Piece Extent=\"0 %d 0 %d 0 %d\">\n", Nx - 1, Ny - 1, Nz - 1);
	x += buf;
	x += "      <PointData>\n";
	for(auto& a : point_data) decl(a, "        ");
	x += "      </PointData>\n      <CellData>\n      </CellData>\n    </Piece>\n  </ImageData>\n";
	x += "  <AppendedData encoding=\"raw\">\n   _";
	bool ok = std::fwrite(x.data(), 1, x.size(), f) == x.size();
	auto put = [&](const VtiArray& a) {
		uint64_t nb = (uint64_t)a.ncomp * a.ntuples * sizeof(double);
		ok = ok && std::fwrite(&nb, sizeof nb, 1, f) == 1;
		ok = ok && (nb == 0 || std::fwrite(a.data, 1, nb, f) == nb);
	};
	for(auto& a : field_data) put(a);
	for(auto& a : point_data) put(a);
	const char* tail = "\n  </AppendedData>\n</VTKFile>\n";
	ok = ok && std::fputs(tail, f) >= 0;
	ok = (std::fclose(f) == 0) && ok;
	return ok ? std::string() : "write error on " + path;
}

// Results folder as PostprocessorBase::format_global_path does (PostprocessorBase.cpp:24-35):
// "<folder>/<base>" with the folder created when it is neither empty nor ".".
inline std::string bulk_output_path(const std::string& folder, const std::string& base) {
	std::string p;
	if(!folder.empty() && folder != ".") {
		::mkdir(folder.c_str(), 0755);
		p = folder + "/";
	}
	return p + base + ".vti";
}

}  // namespace nbpm
