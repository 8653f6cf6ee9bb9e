// hostio.h -- host-side file formats of the NS3D drop-in: the ini input file,
// VTK XML ImageData (.vti) images and fields, and the INFO / RES text logs.
#pragma once

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/ns3d_capi.h"

namespace ns3d {

// ---- ini ----------------------------------------------------------------
struct IniFiles {
    std::string input, pressurefield = "none", vxfield = "none", vyfield = "none", vzfield = "none";
};
// ReadInput (src/navierstokes3D.cxx:266-463): fills p (from defaults) and the
// file keys; messages (warnings and the fatal error) go to `log`.
// Returns false on a fatal error.
bool ini_read(const std::string &path, ns3d_params &p, IniFiles &files, std::string &log);
const char *method_name(int m);

// ---- .vti ---------------------------------------------------------------
struct VtiImage {
    int dims[3] = {0, 0, 0};
    int ncomp = 1;
    std::string type;          // VTK type name of the data array
    std::vector<uint8_t> raw;  // values in file order (x fastest), native bytes
};
bool vti_read(const std::string &path, VtiImage &img, std::string &err);
// values as doubles in file order (x fastest)
bool vti_to_f64(const VtiImage &img, std::vector<double> &out, std::string &err);
// data: nx*ny*nz*ncomp doubles in C order (x slowest, z fastest), written as
// Float64, zlib-compressed appended base64 like the reference's files
bool vti_write_f64(const std::string &path, const double *data, int nx, int ny, int nz, int ncomp,
                   std::string &err);
bool vti_write_u8(const std::string &path, const uint8_t *data_xfastest, int nx, int ny, int nz, std::string &err);

// ---- text logs ------------------------------------------------------------
// std::ostream formatting of the reference: doubles as %.{prec}g
struct TextLog {
    FILE *f = nullptr;
    int prec = 6;
    ~TextLog() { close(); }
    void close() {
        if (f) fclose(f);
        f = nullptr;
    }
    bool open(const std::string &path, int precision) {
        close();
        f = fopen(path.c_str(), "w");
        prec = precision;
        return f != nullptr;
    }
    TextLog &s(const char *t) {
        if (f) fputs(t, f);
        return *this;
    }
    TextLog &s(const std::string &t) { return s(t.c_str()); }
    TextLog &d(double v) {
        if (f) fprintf(f, "%.*g", prec, v);
        return *this;
    }
    TextLog &i(long v) {
        if (f) fprintf(f, "%ld", v);
        return *this;
    }
    void nl() {
        if (f) {
            fputc('\n', f);
            fflush(f);
        }
    }
};

}  // namespace ns3d
