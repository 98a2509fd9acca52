// pp_capture.cpp -- FIXTURE GENERATION ONLY.  Linked with the reference's
// own post-processor (PostProcess.cpp, Derivatives.cpp, VisitWriter.cpp and
// Utils.cpp compiled with its getRange renamed, all read in place), this
// file supplies the getRange(phi, name, Nx, Ny, Nz) that PostProcess.cpp
// calls on every field it computes (PostProcess.cpp:120-308): it writes the
// full FP64 array to "<name>.f64" in the working directory, so that the
// vorticity magnitude and Q-criterion are captured at full precision
// (the program's own output, test.vtk, holds them as float).
#include <cstdio>
#include <string>

void getRange(double *phi, std::string dataName, int Nx, int Ny, int Nz) {
    const std::string path = dataName + ".f64";
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return;
    std::fwrite(phi, sizeof(double), (size_t)Nx * Ny * Nz, f);
    std::fclose(f);
}
