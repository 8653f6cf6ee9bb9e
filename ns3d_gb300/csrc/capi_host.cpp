// capi_host.cpp -- host-only entry points of the C-ABI: ini parsing, .vti I/O
// and the NS3D program (src/navierstokes3D.cxx:480-545) built on the solver
// entry points.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hostio.h"

using namespace ns3d;

static thread_local std::string g_host_err;

static void copy_out(char *dst, const std::string &s, size_t cap) {
    if (!dst || cap == 0) return;
    size_t n = std::min(cap - 1, s.size());
    std::memcpy(dst, s.data(), n);
    dst[n] = 0;
}

// the solver library's error text is per thread; host utilities report there
extern "C" const char *ns3d_last_error(void);

extern "C" {

NS3D_API int ns3d_ini_read(const char *path, ns3d_params *p, char *input, char *pressurefield, char *vxfield,
                           char *vyfield, char *vzfield, size_t cap) {
    if (!path || !p) return NS3D_ERR_ARG;
    IniFiles f;
    std::string log;
    FILE *test = fopen(path, "r");
    if (!test) {
        fprintf(stderr, "error: cannot open input file '%s'\n", path);
        return NS3D_ERR_IO;
    }
    fclose(test);
    bool ok = ini_read(path, *p, f, log);
    if (!log.empty()) fputs(log.c_str(), stderr);
    if (!ok) return NS3D_ERR_PARSE;
    copy_out(input, f.input, cap);
    copy_out(pressurefield, f.pressurefield, cap);
    copy_out(vxfield, f.vxfield, cap);
    copy_out(vyfield, f.vyfield, cap);
    copy_out(vzfield, f.vzfield, cap);
    return NS3D_OK;
}

NS3D_API int ns3d_vti_read_u8(const char *path, uint8_t *buf, size_t cap, int32_t dims[3]) {
    if (!path || !dims) return NS3D_ERR_ARG;
    VtiImage img;
    std::string err;
    if (!vti_read(path, img, err)) {
        fprintf(stderr, "error: %s\n", err.c_str());
        return err.rfind("cannot open", 0) == 0 ? NS3D_ERR_IO : NS3D_ERR_PARSE;
    }
    for (int i = 0; i < 3; ++i) dims[i] = img.dims[i];
    size_t n = (size_t)img.dims[0] * img.dims[1] * img.dims[2];
    if (!buf) return NS3D_OK;
    if (cap < n) return NS3D_ERR_ARG;
    if (img.type == "UInt8" || img.type == "Int8") {
        // the reference reads the scalar buffer as uint8_t (src/vtkio.cxx:130)
        for (size_t i = 0; i < n; ++i) buf[i] = img.raw[i * img.ncomp];
    } else {
        std::vector<double> v;
        if (!vti_to_f64(img, v, err)) return NS3D_ERR_PARSE;
        for (size_t i = 0; i < n; ++i) {
            double x = v[i * img.ncomp];
            buf[i] = (uint8_t)(x < 0 ? 0 : x > 255 ? 255 : (int)x);
        }
    }
    return NS3D_OK;
}

NS3D_API int ns3d_vti_read_f64(const char *path, double *buf, size_t cap, int32_t dims[3], int32_t *ncomp) {
    if (!path || !dims) return NS3D_ERR_ARG;
    VtiImage img;
    std::string err;
    if (!vti_read(path, img, err)) {
        fprintf(stderr, "error: %s\n", err.c_str());
        return err.rfind("cannot open", 0) == 0 ? NS3D_ERR_IO : NS3D_ERR_PARSE;
    }
    for (int i = 0; i < 3; ++i) dims[i] = img.dims[i];
    if (ncomp) *ncomp = img.ncomp;
    if (!buf) return NS3D_OK;
    std::vector<double> v;
    if (!vti_to_f64(img, v, err)) return NS3D_ERR_PARSE;
    if (cap < v.size()) return NS3D_ERR_ARG;
    std::memcpy(buf, v.data(), v.size() * sizeof(double));
    return NS3D_OK;
}

NS3D_API int ns3d_vti_write_f64(const char *path, const double *data, int32_t nx, int32_t ny, int32_t nz,
                                int32_t ncomp) {
    if (!path || !data || nx <= 0 || ny <= 0 || nz <= 0 || ncomp <= 0) return NS3D_ERR_ARG;
    std::string err;
    if (!vti_write_f64(path, data, nx, ny, nz, ncomp, err)) {
        fprintf(stderr, "error: %s\n", err.c_str());
        return NS3D_ERR_IO;
    }
    return NS3D_OK;
}

NS3D_API int ns3d_vti_write_u8(const char *path, const uint8_t *data, int32_t nx, int32_t ny, int32_t nz) {
    if (!path || !data || nx <= 0 || ny <= 0 || nz <= 0) return NS3D_ERR_ARG;
    std::string err;
    if (!vti_write_u8(path, data, nx, ny, nz, err)) {
        fprintf(stderr, "error: %s\n", err.c_str());
        return NS3D_ERR_IO;
    }
    return NS3D_OK;
}

// file order (x fastest) -> C order (x slowest); restart fields are given in
// the solver frame, as the reference reads them (src/NSBase.cxx:2575-2690)
static bool read_field(const std::string &path, int ex, int ny, int nz, std::vector<double> &out) {
    VtiImage img;
    std::string err;
    std::vector<double> v;
    if (!vti_read(path, img, err) || !vti_to_f64(img, v, err)) {
        fprintf(stderr, "error: %s: %s\n", path.c_str(), err.c_str());
        return false;
    }
    if (img.dims[0] != ex || img.dims[1] != ny || img.dims[2] != nz) {
        fprintf(stderr, "error: %s: dimensions %dx%dx%d do not match %dx%dx%d\n", path.c_str(), img.dims[0],
                img.dims[1], img.dims[2], ex, ny, nz);
        return false;
    }
    out.assign((size_t)ex * ny * nz, 0.0);
    for (int x = 0; x < ex; ++x)
        for (int y = 0; y < ny; ++y)
            for (int z = 0; z < nz; ++z)
                out[((size_t)x * ny + y) * nz + z] = v[(((size_t)z * ny + y) * ex + x) * img.ncomp];
    return true;
}

NS3D_API int ns3d_run_ini(const char *ini_path, const char *out_dir, ns3d_result *result) {
    ns3d_params p;
    const size_t cap = 4096;
    std::vector<char> input(cap), pf(cap), vx(cap), vy(cap), vz(cap);
    int rc = ns3d_ini_read(ini_path, &p, input.data(), pf.data(), vx.data(), vy.data(), vz.data(), cap);
    if (rc != NS3D_OK) return rc;
    printf("=== Input parameters ===\n");
    printf("method         : %s\n", method_name(p.method));
    printf("image          : %s\n", input.data());
    printf("dx, dy, dz (m) : %g, %g, %g\n", p.dx, p.dy, p.dz);
    printf("mu (Pa.s)      : %g\n", p.mu);
    printf("rho (kg/m^3)   : %g\n", p.rho);
    printf("p0 (Pa)        : %g\n", p.p0);
    printf("gradp (Pa/m)   : %g\n", p.gradp);
    printf("alpha, beta    : %g, %g\n", p.alpha, p.beta);
    printf("simpletol      : %g\n", p.simpletol);
    printf("maxitSIMPLE    : %d\n", p.maxitSIMPLE);
    printf("maxitsolver    : %d\n", p.maxitsolver);
    printf("save_step      : %d\n", p.save_step);
    printf("porevalue      : %d\n", p.porevalue);
    printf("direction      : %d\n", p.direction);
    printf("border         : %d\n", p.border);
    printf("======================\n");
    int32_t dims[3];
    rc = ns3d_vti_read_u8(input.data(), nullptr, 0, dims);
    if (rc != NS3D_OK) return rc;
    std::vector<uint8_t> raw((size_t)dims[0] * dims[1] * dims[2]);
    rc = ns3d_vti_read_u8(input.data(), raw.data(), raw.size(), dims);
    if (rc != NS3D_OK) return rc;
    ns3d_handle *h = nullptr;
    rc = ns3d_open(&p, raw.data(), dims[0], dims[1], dims[2], &h);
    if (rc != NS3D_OK) {
        fprintf(stderr, "error: %s\n", ns3d_last_error());
        return rc;
    }
    ns3d_sizes s;
    ns3d_get_sizes(h, &s);
    printf("Size %d, %d, %d\n", s.nx, s.ny, s.nz);
    printf("Porosity: %g\n", (double)(float(s.np) / float((long)s.nx * s.ny * s.nz)));
    printf("Nodes for the pressure field: %d\n", s.np);
    printf("Nodes for the u velocity field: %d\n", s.nu);
    printf("Nodes for the v velocity field: %d\n", s.nv);
    printf("Nodes for the w velocity field: %d\n", s.nw);
    std::vector<double> fp, fu, fv, fw;
    bool ok = true;
    if (std::string(pf.data()) != "none") ok = ok && read_field(pf.data(), s.nx, s.ny, s.nz, fp);
    if (std::string(vx.data()) != "none") ok = ok && read_field(vx.data(), s.nx + 1, s.ny, s.nz, fu);
    if (std::string(vy.data()) != "none") ok = ok && read_field(vy.data(), s.nx, s.ny, s.nz, fv);
    if (std::string(vz.data()) != "none") ok = ok && read_field(vz.data(), s.nx, s.ny, s.nz, fw);
    if (!ok) {
        ns3d_close(h);
        return NS3D_ERR_IO;
    }
    rc = ns3d_set_initial_fields(h, fp.empty() ? nullptr : fp.data(), fu.empty() ? nullptr : fu.data(),
                                 fv.empty() ? nullptr : fv.data(), fw.empty() ? nullptr : fw.data());
    // outputs are named after the image: basename with the last 4 characters
    // removed (src/NSBase.cxx:107-117)
    std::string img = input.data();
    size_t slash = img.find_last_of('/');
    if (slash != std::string::npos) img.erase(0, slash + 1);
    std::string stem = img.size() >= 4 ? img.substr(0, img.size() - 4) : img;
    if (rc == NS3D_OK) rc = ns3d_set_output(h, out_dir ? out_dir : ".", stem.c_str(), 1);
    if (rc == NS3D_OK) rc = ns3d_solve(h);
    if (rc != NS3D_OK) {
        fprintf(stderr, "error: %s\n", ns3d_last_error());
        ns3d_close(h);
        return rc;
    }
    ns3d_result r;
    ns3d_get_result(h, &r);
    printf("Permeability K (m²): %g\n", r.K);
    printf("%s terminated in %d iteration and %g seconds\n", method_name(p.method), r.iterations, r.seconds);
    if (result) *result = r;
    ns3d_close(h);
    return NS3D_OK;
}

}  // extern "C"
