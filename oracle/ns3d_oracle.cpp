/*
 * ns3d_oracle.cpp -- CPU restatement of the NS3D permeability solve.
 *
 * TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.  Only tests/, the smoke()
 * entry and bench.py's CPU-baseline leg load this library; the CUDA library
 * never links or calls it.
 *
 * It restates, loop by loop and with the floating-point expression order of
 * the reference kept, the solver of jerome-lux/NS3D:
 *   src/NSBase.cxx   geometry, index arrays, assembly, corrections,
 *                    diagnostics, relaxation control (cited per function)
 *   src/SIMPLEC.cxx, src/SIMPLER.cxx, src/SIMPLERR.cxx, src/IDEAL.cxx
 *                    the four outer loops
 *   src/vtkio.cxx:96-150   binarization and axis order of the input image
 * and implements include/ns3d_capi.h so it can be swapped with the CUDA
 * library.
 *
 * The linear solver of the reference is Eigen 3.x BiCGSTAB with the default
 * DiagonalPreconditioner (src/NSBase.h:97-100; Eigen is not vendored, its
 * version is unpinned, README.md:54 asks for >= 3.3).  It is restated here
 * from the published algorithm (van der Vorst 1992, right-preconditioned)
 * with the behaviour the reference relies on: convergence when
 * |r|^2 <= tol^2 |b|^2, iterations() = completed iterations,
 * error() = |r|/|b|, a restart with a fresh shadow residual when
 * |rho| < eps^2 |r0|^2 (the iteration counter restarts on the first one), a
 * zero diagonal preconditioned by 1, and the zero right-hand-side rule
 * (x = 0, Success, iterations() left at the maximum) that the golden INFO log
 * shows as "500 iterations (status 0)".
 *
 * Summation order.  Eigen's SIMD reduction order cannot be reproduced, so
 * every floating-point sum over rows here uses one fixed, documented order
 * (det_sum below) that the CUDA kernels reproduce exactly: rows are cut into
 * chunks of 1024; inside a chunk, lane l (0..127) accumulates rows
 * l, l+128, ..., l+896 in order; the lanes of each group of 32 are combined
 * by a halving tree (offsets 16,8,4,2,1), then the 4 group sums by a halving
 * tree (offsets 2,1); chunk partials are combined the same way (lane l
 * sums partials l, l+128, ... in order, then the trees).  Sparse rows are
 * summed in ascending column order (Eigen's compressed row-major storage).
 * Fused multiply-adds appear only where written as std::fma; the file is
 * built with -ffp-contract=off so every other expression rounds as written.
 * With these rules the CUDA path can match this oracle bit for bit.
 */
#include "../include/ns3d_capi.h"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <list>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

/* ---------------- fixed-order reductions -------------------------------- */
constexpr long CH = 1024;   // rows per chunk
constexpr int LANES = 128;  // lanes per chunk
constexpr int RPL = 8;      // rows per lane, strided by LANES

inline double tree_sum(double *a) {
    double w[LANES / 32];
    for (int g = 0; g < LANES / 32; ++g) {
        double *b = a + 32 * g;
        for (int off = 16; off >= 1; off >>= 1)
            for (int l = 0; l < off; ++l) b[l] = b[l] + b[l + off];
        w[g] = b[0];
    }
    for (int off = LANES / 64; off >= 1; off >>= 1)
        for (int l = 0; l < off; ++l) w[l] = w[l] + w[l + off];
    return w[0];
}

inline double final_sum(const std::vector<double> &part) {
    double acc[LANES];
    for (int l = 0; l < LANES; ++l) {
        double a = 0.0;
        for (size_t i = (size_t)l; i < part.size(); i += LANES) a = a + part[i];
        acc[l] = a;
    }
    return tree_sum(acc);
}

/* f(row, acc) returns the new lane accumulator */
template <class F>
double det_sum(long n, F f) {
    long nch = (n + CH - 1) / CH;
    std::vector<double> part((size_t)nch);
#pragma omp parallel for schedule(static)
    for (long c = 0; c < nch; ++c) {
        double acc[LANES];
        for (int l = 0; l < LANES; ++l) {
            double a = 0.0;
            for (int m = 0; m < RPL; ++m) {
                long r = c * CH + (long)l + (long)LANES * m;
                if (r < n) a = f(r, a);
            }
            acc[l] = a;
        }
        part[(size_t)c] = tree_sum(acc);
    }
    return final_sum(part);
}

double det_dot(const std::vector<double> &a, const std::vector<double> &b, long n) {
    const double *pa = a.data(), *pb = b.data();
    return det_sum(n, [&](long r, double acc) { return std::fma(pa[r], pb[r], acc); });
}

/*
 * Alternative rounding of the BiCGSTAB arithmetic, for experiments only
 * (environment variable NS3D_ORACLE_ARITH, read when a solver opens; unset
 * or "fixed" = the documented contract above, which the CUDA path follows):
 *   "serial"   every product rounded before its add, dot products summed
 *              row 0..n-1 with one accumulator, sparse rows in ascending
 *              column order (what a scalar build of a sparse library does)
 *   "packet4"  as "serial" but dot products with 4 interleaved accumulators
 *              combined pairwise at the end (a 4-wide SIMD reduction)
 * They exist to measure how much a solve's trajectory depends on rounding
 * alone (the reference's Eigen reduction order cannot be reproduced).
 */
// Wall time per phase since the last ns3d_solve started, process-wide (the
// CPU baseline runs one solve per process and reports it beside the total):
// 0 assembly (momentum, right-hand sides, pseudo-velocities, pressure
// systems), 1 BiCGSTAB solves, 2 corrections, 3 diagnostics (permeability,
// divergence).
double g_phase_s[4] = {0, 0, 0, 0};
struct PhaseTimer {
    int slot;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    explicit PhaseTimer(int s) : slot(s) {}
    ~PhaseTimer() {
        g_phase_s[slot] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

int g_arith = 0;

void read_arith_mode() {
    const char *e = getenv("NS3D_ORACLE_ARITH");
    g_arith = 0;
    if (e && !strcmp(e, "serial")) g_arith = 1;
    else if (e && !strcmp(e, "packet4")) g_arith = 2;
}

double alt_dot(const std::vector<double> &a, const std::vector<double> &b, long n) {
    if (g_arith == 1) {
        double acc = 0.0;
        for (long r = 0; r < n; ++r) acc = acc + a[(size_t)r] * b[(size_t)r];
        return acc;
    }
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    long r = 0;
    for (; r + 4 <= n; r += 4)
        for (int k = 0; k < 4; ++k) acc[k] = acc[k] + a[(size_t)(r + k)] * b[(size_t)(r + k)];
    double t = (acc[0] + acc[2]) + (acc[1] + acc[3]);
    for (; r < n; ++r) t = t + a[(size_t)r] * b[(size_t)r];
    return t;
}

inline double bdot(const std::vector<double> &a, const std::vector<double> &b, long n) {
    return g_arith == 0 ? det_dot(a, b, n) : alt_dot(a, b, n);
}

/* std::min(F,0.0) / std::max(F,0.0) exactly as the standard library selects */
inline double min0(double F) { return (0.0 < F) ? 0.0 : F; }
inline double max0(double F) { return (F < 0.0) ? 0.0 : F; }

/* ---------------- sparse systems ---------------------------------------- */
enum { SP = 0, SW = 1, SE = 2, SS = 3, SN = 4, SB = 5, ST = 6 };

struct System {
    int n = 0;
    int d0 = 0;                   // first extent of the index map (nx or nx+1)
    std::vector<int> cell;        // row -> linear position in its index map
    std::vector<double> c[7];     // coefficients per slot P,W,E,S,N,B,T
    std::vector<int> nb[6];       // column per off-diagonal slot (-1 none)
    std::vector<double> rhs, rowsum, invdiag;
    // compressed rows, columns ascending (Eigen's storage order)
    std::vector<int> rp, col, slot;

    void resize(int nn) {
        n = nn;
        for (auto &v : c) v.assign((size_t)n, 0.0);
        for (auto &v : nb) v.assign((size_t)n, -1);
        rhs.assign((size_t)n, 0.0);
        rowsum.assign((size_t)n, 0.0);
        invdiag.assign((size_t)n, 1.0);
    }
    // pattern -> ascending-column entry list per row
    void build_pattern() {
        rp.assign((size_t)n + 1, 0);
        for (int r = 0; r < n; ++r) {
            int cnt = 1;
            for (int s = 0; s < 6; ++s) cnt += nb[s][(size_t)r] >= 0;
            rp[(size_t)r + 1] = rp[(size_t)r] + cnt;
        }
        col.assign((size_t)rp[(size_t)n], 0);
        slot.assign((size_t)rp[(size_t)n], 0);
#pragma omp parallel for schedule(static)
        for (int r = 0; r < n; ++r) {
            int cs[7], ss[7], m = 0;
            cs[m] = r; ss[m] = SP; ++m;
            for (int s = 0; s < 6; ++s) {
                int cc = nb[s][(size_t)r];
                if (cc >= 0) { cs[m] = cc; ss[m] = s + 1; ++m; }
            }
            for (int a = 1; a < m; ++a)  // insertion sort by column
                for (int b = a; b > 0 && cs[b - 1] > cs[b]; --b) {
                    std::swap(cs[b - 1], cs[b]);
                    std::swap(ss[b - 1], ss[b]);
                }
            int o = rp[(size_t)r];
            for (int a = 0; a < m; ++a) { col[(size_t)o + a] = cs[a]; slot[(size_t)o + a] = ss[a]; }
        }
    }
    inline double val(int e, int r) const { return c[slot[(size_t)e]][(size_t)r]; }
    // y = A x, each row summed with fma in ascending column order
    void spmv(const std::vector<double> &x, std::vector<double> &y) const {
        if (g_arith != 0) {  // experiments: products rounded before the adds
#pragma omp parallel for schedule(static)
            for (int r = 0; r < n; ++r) {
                double t = 0.0;
                for (int e = rp[(size_t)r]; e < rp[(size_t)r + 1]; ++e) t = t + val(e, r) * x[(size_t)col[(size_t)e]];
                y[(size_t)r] = t;
            }
            return;
        }
#pragma omp parallel for schedule(static)
        for (int r = 0; r < n; ++r) {
            double t = 0.0;
            for (int e = rp[(size_t)r]; e < rp[(size_t)r + 1]; ++e) t = std::fma(val(e, r), x[(size_t)col[(size_t)e]], t);
            y[(size_t)r] = t;
        }
    }
    // uA.row(r).sum(): stored entries in storage order, plain adds from 0
    void compute_rowsum() {
#pragma omp parallel for schedule(static)
        for (int r = 0; r < n; ++r) {
            double t = 0.0;
            for (int e = rp[(size_t)r]; e < rp[(size_t)r + 1]; ++e) t = t + val(e, r);
            rowsum[(size_t)r] = t;
        }
    }
    // Jacobi: 1/a_rr, or 1 when the diagonal is 0
    void compute_invdiag() {
#pragma omp parallel for schedule(static)
        for (int r = 0; r < n; ++r) {
            double d = c[SP][(size_t)r];
            invdiag[(size_t)r] = (d != 0.0) ? 1.0 / d : 1.0;
        }
    }
};

struct SolveOut {
    long iters = 0;
    long work = 0;  // iterations executed, restarts included
    double error = 0.0;
    int info = NS3D_SUCCESS;
    bool valid = false;
};

/*
 * Right-preconditioned BiCGSTAB (van der Vorst), Eigen semantics (see the
 * file header).  Element updates:
 *   p = r + beta (p - w v)      as fma(beta, fma(-w, v, p), r)
 *   s = r - alpha v             as fma(-alpha, v, r)
 *   x = x + alpha y + w z       as fma(w, z, fma(alpha, y, x))
 *   r = s - w t                 as fma(-w, t, s)
 */
SolveOut bicgstab(const System &A, const std::vector<double> &b, std::vector<double> &x,
                  double tol, long maxit, long *krylov_rows) {
    PhaseTimer phase_timer(1);
    const long n = A.n;
    SolveOut out;
    out.valid = true;
    std::vector<double> r((size_t)n), r0, p((size_t)n, 0.0), v((size_t)n, 0.0), y((size_t)n), z((size_t)n),
        s((size_t)n), t((size_t)n), ax((size_t)n);
    A.spmv(x, ax);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) r[(size_t)i] = b[(size_t)i] - ax[(size_t)i];
    r0 = r;
    double r0_sqnorm = bdot(r0, r0, n);
    double rhs_sqnorm = bdot(b, b, n);
    if (rhs_sqnorm == 0.0) {
        std::fill(x.begin(), x.end(), 0.0);
        out.iters = maxit;
        out.error = tol;
        out.info = NS3D_SUCCESS;
        return out;
    }
    double rho = 1.0, alpha = 1.0, w = 1.0;
    const double tol2 = tol * tol * rhs_sqnorm;
    const double eps2 = DBL_EPSILON * DBL_EPSILON;
    long i = 0;
    int restarts = 0;
    double rr = bdot(r, r, n);
    const double *iv = A.invdiag.data();
    while (rr > tol2 && i < maxit) {
        double rho_old = rho;
        rho = bdot(r0, r, n);
        if (std::fabs(rho) < eps2 * r0_sqnorm) {
            A.spmv(x, ax);
#pragma omp parallel for schedule(static)
            for (long k = 0; k < n; ++k) r[(size_t)k] = b[(size_t)k] - ax[(size_t)k];
            r0 = r;
            rho = r0_sqnorm = bdot(r, r, n);
            if (restarts++ == 0) i = 0;
        }
        double beta = (rho / rho_old) * (alpha / w);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < n; ++k) {
            double pk = g_arith ? r[(size_t)k] + beta * (p[(size_t)k] - w * v[(size_t)k])
                                : std::fma(beta, std::fma(-w, v[(size_t)k], p[(size_t)k]), r[(size_t)k]);
            p[(size_t)k] = pk;
            y[(size_t)k] = iv[k] * pk;
        }
        A.spmv(y, v);
        alpha = rho / bdot(r0, v, n);
#pragma omp parallel for schedule(static)
        for (long k = 0; k < n; ++k) {
            double sk = g_arith ? r[(size_t)k] - alpha * v[(size_t)k] : std::fma(-alpha, v[(size_t)k], r[(size_t)k]);
            s[(size_t)k] = sk;
            z[(size_t)k] = iv[k] * sk;
        }
        A.spmv(z, t);
        double tmp = bdot(t, t, n);
        double ts = bdot(t, s, n);
        if (tmp > 0.0)
            w = ts / tmp;
        else
            w = 0.0;
#pragma omp parallel for schedule(static)
        for (long k = 0; k < n; ++k) {
            if (g_arith) {
                x[(size_t)k] = x[(size_t)k] + (alpha * y[(size_t)k] + w * z[(size_t)k]);
                r[(size_t)k] = s[(size_t)k] - w * t[(size_t)k];
            } else {
                x[(size_t)k] = std::fma(w, z[(size_t)k], std::fma(alpha, y[(size_t)k], x[(size_t)k]));
                r[(size_t)k] = std::fma(-w, t[(size_t)k], s[(size_t)k]);
            }
        }
        rr = bdot(r, r, n);
        ++i;
        ++out.work;
        if (krylov_rows) *krylov_rows += n;
    }
    out.iters = i;
    out.error = std::sqrt(rr / rhs_sqnorm);
    out.info = (out.error <= tol) ? NS3D_SUCCESS : NS3D_NO_CONVERGENCE;
    return out;
}

/* ---------------- text logs ---------------------------------------------- */
struct Log {
    FILE *f = nullptr;
    int prec = 6;
    ~Log() { close(); }
    void close() {
        if (f) fclose(f);
        f = nullptr;
    }
    void s(const char *t) { if (f) fputs(t, f); }
    void d(double v) { if (f) fprintf(f, "%.*g", prec, v); }
    void i(long v) { if (f) fprintf(f, "%ld", v); }
    void nl() { if (f) { fputc('\n', f); fflush(f); } }
};

/* ---------------- solver instance --------------------------------------- */
struct Handle {
    ns3d_params prm;
    int nx = 0, ny = 0, nz = 0;
    int np = 0, nu = 0, nv = 0, nw = 0;
    std::vector<int> pindex, uindex, vindex, windex;
    System U, V, W, P;  // momentum systems and the pressure(-correction) system

    double dx, dy, dz, mu, rho, p0, p1, gradp, alpha0, beta0, alpha, beta;
    double p_inlet = 0, p_outlet = 0;
    double schemefactor, min_alpha, min_beta, relax, speedup, maxconvdelta;
    double RMR = 0, old_RMR = 0, deltaRMR;
    double pcmax = 0, pcmin = 0, pcnorm = 0;
    std::list<double> avgRMR;
    int border;

    std::vector<double> p, u, v, w, pc;
    bool fields_ready = false;
    SolveOut su, sv, sw, sp;
    ns3d_result res;

    std::string outdir, stem;
    bool have_out = false;
    Log info, resl;

    // linear positions in the maps
    inline long pid(int i, int j, int k) const { return ((long)i * ny + j) * nz + k; }
    inline long uid(int i, int j, int k) const { return ((long)i * ny + j) * nz + k; }  // i in [0,nx]
    inline int Pm(int i, int j, int k) const { return pindex[(size_t)pid(i, j, k)]; }
    inline int Um(int i, int j, int k) const { return uindex[(size_t)uid(i, j, k)]; }
    inline int Vm(int i, int j, int k) const { return vindex[(size_t)pid(i, j, k)]; }
    inline int Wm(int i, int j, int k) const { return windex[(size_t)pid(i, j, k)]; }

    // SafeVectorValue, src/NSBase.cxx:1757-1771
    inline double Su(const std::vector<double> &f, int i, int j, int k) const {
        if (i >= nx + 1 || i < 0 || j >= ny || j < 0 || k >= nz || k < 0) return 0;
        int r = Um(i, j, k);
        return r > -1 ? f[(size_t)r] : 0;
    }
    inline double Sv(const std::vector<double> &f, int i, int j, int k) const {
        if (i >= nx || i < 0 || j >= ny || j < 0 || k >= nz || k < 0) return 0;
        int r = Vm(i, j, k);
        return r > -1 ? f[(size_t)r] : 0;
    }
    inline double Sw(const std::vector<double> &f, int i, int j, int k) const {
        if (i >= nx || i < 0 || j >= ny || j < 0 || k >= nz || k < 0) return 0;
        int r = Wm(i, j, k);
        return r > -1 ? f[(size_t)r] : 0;
    }
    inline void ijk(long lin, int &i, int &j, int &k) const {
        k = (int)(lin % nz);
        long t = lin / nz;
        j = (int)(t % ny);
        i = (int)(t / ny);
    }
};

/* ---- geometry: src/vtkio.cxx:96-150, src/NSBase.cxx:2425-2573 ----------- */
int build_geometry(Handle &h, const uint8_t *raw, int rnx, int rny, int rnz) {
    const ns3d_params &q = h.prm;
    // binarize, VTK x-fastest -> C order (x,y,z), z fastest
    std::vector<uint8_t> img((size_t)rnx * rny * rnz);
    const uint8_t pv = (uint8_t)q.porevalue;
    for (int x = 0; x < rnx; ++x)
        for (int y = 0; y < rny; ++y)
            for (int z = 0; z < rnz; ++z)
                img[((size_t)x * rny + y) * rnz + z] = (raw[((size_t)z * rny + y) * rnx + x] == pv) ? 0 : 1;
    int ax = rnx, ay = rny, az = rnz;
    // Rotation, src/NSBase.cxx:2451-2492
    if (q.direction == 2) {
        std::vector<uint8_t> t((size_t)ay * ax * az);
        for (int i = 0; i < ax; ++i)
            for (int j = 0; j < ay; ++j)
                for (int k = 0; k < az; ++k)
                    t[((size_t)j * ax + (ax - 1 - i)) * az + k] = img[((size_t)i * ay + j) * az + k];
        img.swap(t);
        std::swap(ax, ay);
    } else if (q.direction == 3) {
        std::vector<uint8_t> t((size_t)az * ay * ax);
        for (int i = 0; i < ax; ++i)
            for (int j = 0; j < ay; ++j)
                for (int k = 0; k < az; ++k)
                    t[((size_t)k * ay + j) * ax + i] = img[((size_t)i * ay + j) * az + k];
        img.swap(t);
        std::swap(ax, az);
    }
    // AddBorder pads with 0 (= fluid), src/NSBase.cxx:2425-2448
    if (q.border > 0) {
        int b = q.border;
        std::vector<uint8_t> t((size_t)(ax + 2 * b) * ay * az, 0);
        for (int i = 0; i < ax; ++i)
            std::memcpy(&t[(size_t)(i + b) * ay * az], &img[(size_t)i * ay * az], (size_t)ay * az);
        img.swap(t);
        ax += 2 * b;
    }
    h.nx = ax; h.ny = ay; h.nz = az;
    const int nx = ax, ny = ay, nz = az;
    const size_t N = (size_t)nx * ny * nz;
    h.pindex.assign(N, -1);
    h.vindex.assign(N, -1);
    h.windex.assign(N, -1);
    h.uindex.assign((size_t)(nx + 1) * ny * nz, -1);
    // InitIndexArrays, src/NSBase.cxx:2495-2573 (sequential numbering)
    int np = -1, nu = -1, nv = -1, nw = -1;
    auto I = [&](int i, int j, int k) { return (int)img[((size_t)i * ny + j) * nz + k]; };
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                if (I(i, j, k) != 0) continue;
                bool has = false;
                size_t c = ((size_t)i * ny + j) * nz + k;
                if (j > 0 && I(i, j - 1, k) == 0) { h.vindex[c] = ++nv; has = true; }
                if (j < ny - 1 && I(i, j + 1, k) == 0) has = true;
                if (k > 0 && I(i, j, k - 1) == 0) { h.windex[c] = ++nw; has = true; }
                if (nz > 0 && k < nz - 1 && I(i, j, k + 1) == 0) has = true;
                if (i == 0) { h.uindex[c] = ++nu; has = true; }
                if (i > 0 && I(i - 1, j, k) == 0) { h.uindex[c] = ++nu; has = true; }
                if (i == nx - 1) { h.uindex[((size_t)nx * ny + j) * nz + k] = ++nu; has = true; }
                if (i < nx - 1 && I(i + 1, j, k) == 0) has = true;
                if (has) h.pindex[c] = ++np;
            }
    h.np = np + 1; h.nu = nu + 1; h.nv = nv + 1; h.nw = nw + 1;
    return NS3D_OK;
}

/* row -> cell tables and sparsity patterns of the four systems */
void build_systems(Handle &h) {
    const int nx = h.nx, ny = h.ny, nz = h.nz;
    auto setup = [&](System &S, const std::vector<int> &map, int d0, int n) {
        S.resize(n);
        S.d0 = d0;
        S.cell.assign((size_t)n, 0);
        for (long c = 0; c < (long)map.size(); ++c)
            if (map[(size_t)c] > -1) S.cell[(size_t)map[(size_t)c]] = (int)c;
    };
    setup(h.U, h.uindex, nx + 1, h.nu);
    setup(h.V, h.vindex, nx, h.nv);
    setup(h.W, h.windex, nx, h.nw);
    setup(h.P, h.pindex, nx, h.np);
    // momentum patterns: an entry for every neighbour node of the same map
    // (k-direction only when the image has more than one z layer)
    auto mom = [&](System &S, const std::vector<int> &map, bool zdir) {
        const int d0 = S.d0;
#pragma omp parallel for schedule(static)
        for (int r = 0; r < S.n; ++r) {
            long c = S.cell[(size_t)r];
            int k = (int)(c % nz), j = (int)((c / nz) % ny), i = (int)(c / ((long)ny * nz));
            auto M = [&](int a, int b, int cc) { return map[((size_t)a * ny + b) * nz + cc]; };
            S.nb[0][(size_t)r] = (i - 1 >= 0) ? M(i - 1, j, k) : -1;
            S.nb[1][(size_t)r] = (i + 1 < d0) ? M(i + 1, j, k) : -1;
            S.nb[2][(size_t)r] = (j - 1 >= 0) ? M(i, j - 1, k) : -1;
            S.nb[3][(size_t)r] = (j + 1 < ny) ? M(i, j + 1, k) : -1;
            S.nb[4][(size_t)r] = (zdir && k - 1 >= 0) ? M(i, j, k - 1) : -1;
            S.nb[5][(size_t)r] = (zdir && k + 1 < nz) ? M(i, j, k + 1) : -1;
        }
        S.build_pattern();
    };
    mom(h.U, h.uindex, nz > 1);
    mom(h.V, h.vindex, nz > 1);
    mom(h.W, h.windex, true);
    // pressure pattern: neighbour node and the face node between them
    System &S = h.P;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < S.n; ++r) {
        int i, j, k;
        h.ijk(S.cell[(size_t)r], i, j, k);
        S.nb[0][(size_t)r] = (i > 0 && h.Pm(i - 1, j, k) > -1 && h.Um(i, j, k) > -1) ? h.Pm(i - 1, j, k) : -1;
        S.nb[1][(size_t)r] = (i < nx - 1 && h.Pm(i + 1, j, k) > -1 && h.Um(i + 1, j, k) > -1) ? h.Pm(i + 1, j, k) : -1;
        S.nb[2][(size_t)r] = (j > 0 && h.Pm(i, j - 1, k) > -1 && h.Vm(i, j, k) > -1) ? h.Pm(i, j - 1, k) : -1;
        S.nb[3][(size_t)r] = (j < ny - 1 && h.Pm(i, j + 1, k) > -1 && h.Vm(i, j + 1, k) > -1) ? h.Pm(i, j + 1, k) : -1;
        S.nb[4][(size_t)r] = (k > 0 && nz > 0 && h.Pm(i, j, k - 1) > -1 && h.Wm(i, j, k) > -1) ? h.Pm(i, j, k - 1) : -1;
        S.nb[5][(size_t)r] = (k < nz - 1 && nz > 0 && h.Pm(i, j, k + 1) > -1 && h.Wm(i, j, k + 1) > -1) ? h.Pm(i, j, k + 1) : -1;
    }
    S.build_pattern();
}

/* ---- momentum assembly: src/NSBase.cxx:886-1442 ------------------------- */
void assemble_mom_x(Handle &h, const std::vector<double> &uc, const std::vector<double> &vc,
                    const std::vector<double> &wc) {
    System &A = h.U;
    const double dx = h.dx, dy = h.dy, dz = h.dz, mu = h.mu, rho = h.rho, sf = h.schemefactor;
    const double idx2 = 1 / (dx * dx), idy2 = 1 / (dy * dy), idz2 = 1 / (dz * dz);
    const double idx = 1 / dx, idy = 1 / dy, idz = 1 / dz;
    const int d0 = h.nx + 1, ny = h.ny, nz = h.nz;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < A.n; ++r) {
        int i, j, k;
        h.ijk(A.cell[(size_t)r], i, j, k);
        double D = 0, F, um, vm, wm, Fd;
        double aW = 0, aE = 0, aS = 0, aN = 0, aB = 0, aT = 0;
        double uC = h.Su(uc, i, j, k);
        if (i + 1 < d0) {
            if (h.Um(i + 1, j, k) > -1) {
                double uE = h.Su(uc, i + 1, j, k);
                if (uC > 0 && uE > 0) F = -uC * rho * idx;
                else if (uC < 0 && uE < 0) F = -uE * rho * idx;
                else F = 0;
                if (std::fabs(F) * dx * dx > 2 * mu * sf) {
                    D += -mu * idx2 + min0(F);
                    aE = mu * idx2 + max0(F);
                } else {
                    um = (uC + uE) * 0.5;
                    Fd = -um * rho * idx;
                    D += -mu * idx2 + Fd * 0.5;
                    aE = mu * idx2 + Fd * 0.5;
                }
            } else {
                D += -mu * idx2 - (0.25 * rho * idx) * (uC);
            }
        } else {
            D += -(rho * idx) * (uC);
        }
        if (i - 1 >= 0) {
            if (h.Um(i - 1, j, k) > -1) {
                double uW = h.Su(uc, i - 1, j, k);
                if (uC < 0 && uW < 0) F = uC * rho * idx;
                else if (uC > 0 && uW > 0) F = uW * rho * idx;
                else F = 0;
                if (std::fabs(F) * dx * dx > 2 * mu * sf) {
                    D += -mu * idx2 + min0(F);
                    aW = mu * idx2 + max0(F);
                } else {
                    um = (uC + uW) * 0.5;
                    Fd = um * rho * idx;
                    D += -mu * idx2 + Fd * 0.5;
                    aW = mu * idx2 + Fd * 0.5;
                }
            } else {
                D += -mu * idx2 + (0.25 * rho * idx) * (uC);
            }
        } else {
            D += (rho * idx) * (uC);
        }
        if (j + 1 < ny) {
            if (h.Um(i, j + 1, k) > -1) {
                vm = (h.Sv(vc, i - 1, j + 1, k) + h.Sv(vc, i, j + 1, k)) * 0.5;
                F = -vm * rho * idy;
                if (std::fabs(vm) * rho * dy > 2 * mu * sf) {
                    D += -mu * idy2 + min0(F);
                    aN = mu * idy2 + max0(F);
                } else {
                    D += -mu * idy2 + F * 0.5;
                    aN = mu * idy2 + F * 0.5;
                }
            } else {
                D += -2 * mu * idy2;
            }
        } else {
            D += -2 * mu * idy2;
        }
        if (j - 1 >= 0) {
            if (h.Um(i, j - 1, k) > -1) {
                vm = (h.Sv(vc, i - 1, j, k) + h.Sv(vc, i, j, k)) * 0.5;
                F = vm * rho * idy;
                if (std::fabs(vm) * dy * rho > 2 * mu * sf) {
                    D += -mu * idy2 + min0(F);
                    aS = mu * idy2 + max0(F);
                } else {
                    D += -mu * idy2 + F * 0.5;
                    aS = mu * idy2 + F * 0.5;
                }
            } else {
                D += -2 * mu * idy2;
            }
        } else {
            D += -2 * mu * idy2;
        }
        if (nz > 1) {
            if (k + 1 < nz) {
                if (h.Um(i, j, k + 1) > -1) {
                    wm = (h.Sw(wc, i - 1, j, k + 1) + h.Sw(wc, i, j, k + 1)) * 0.5;
                    F = -wm * rho * idz;
                    if (std::fabs(wm) * rho * dz > 2 * mu * sf) {
                        D += -mu * idz2 + min0(F);
                        aT = mu * idz2 + max0(F);
                    } else {
                        D += -mu * idz2 + F * 0.5;
                        aT = mu * idz2 + F * 0.5;
                    }
                } else {
                    D += -2 * mu * idz2;
                }
            } else {
                D += -2 * mu * idz2;
            }
            if (k - 1 >= 0) {
                if (h.Um(i, j, k - 1) > -1) {
                    wm = (h.Sw(wc, i - 1, j, k) + h.Sw(wc, i, j, k)) * 0.5;
                    F = wm * rho * idz;
                    if (std::fabs(wm) * rho * dz > 2 * mu * sf) {
                        D += -mu * idz2 + min0(F);
                        aB = mu * idz2 + max0(F);
                    } else {
                        D += -mu * idz2 + F * 0.5;
                        aB = mu * idz2 + F * 0.5;
                    }
                } else {
                    D += -2 * mu * idz2;
                }
            } else {
                D += -2 * mu * idz2;
            }
        }
        D /= h.alpha;
        A.c[SP][(size_t)r] = D;
        A.c[SW][(size_t)r] = aW; A.c[SE][(size_t)r] = aE;
        A.c[SS][(size_t)r] = aS; A.c[SN][(size_t)r] = aN;
        A.c[SB][(size_t)r] = aB; A.c[ST][(size_t)r] = aT;
    }
}

void assemble_mom_y(Handle &h, const std::vector<double> &uc, const std::vector<double> &vc,
                    const std::vector<double> &wc) {
    System &A = h.V;
    const double dx = h.dx, dy = h.dy, dz = h.dz, mu = h.mu, rho = h.rho, sf = h.schemefactor;
    const double idx2 = 1 / (dx * dx), idy2 = 1 / (dy * dy), idz2 = 1 / (dz * dz);
    const double idx = 1 / dx, idy = 1 / dy, idz = 1 / dz;
    const int d0 = h.nx, ny = h.ny, nz = h.nz;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < A.n; ++r) {
        int i, j, k;
        h.ijk(A.cell[(size_t)r], i, j, k);
        double D = 0, F, um, vm, wm, Fd;
        double aW = 0, aE = 0, aS = 0, aN = 0, aB = 0, aT = 0;
        if (i + 1 < d0) {
            if (h.Vm(i + 1, j, k) > -1) {
                um = (h.Su(uc, i + 1, j - 1, k) + h.Su(uc, i + 1, j, k)) * 0.5;
                F = -um * rho * idx;
                if (std::fabs(um) * dx * rho > 2 * mu * sf) {
                    D += -mu * idx2 + min0(F);
                    aE = mu * idx2 + max0(F);
                } else {
                    D += -mu * idx2 + F * 0.5;
                    aE = mu * idx2 + F * 0.5;
                }
            } else {
                D += -2 * mu * idx2;
            }
        } else {
            D += -(0.5 * rho * idx) * (h.Su(uc, i + 1, j - 1, k) + h.Su(uc, i + 1, j, k));
        }
        if (i - 1 >= 0) {
            if (h.Vm(i - 1, j, k) > -1) {
                um = (h.Su(uc, i, j - 1, k) + h.Su(uc, i, j, k)) * 0.5;
                F = um * rho * idx;
                if (std::fabs(um) * dx * rho > 2 * mu * sf) {
                    D += -mu * idx2 + min0(F);
                    aW = mu * idx2 + max0(F);
                } else {
                    D += -mu * idx2 + F * 0.5;
                    aW = mu * idx2 + F * 0.5;
                }
            } else {
                D += -2 * mu * idx2;
            }
        } else {
            D += -mu * idx2 + (0.25 * rho * idx) * (h.Su(uc, i, j - 1, k) + h.Su(uc, i, j, k));
        }
        double vC = h.Sv(vc, i, j, k);
        if (j + 1 < ny) {
            if (h.Vm(i, j + 1, k) > -1) {
                double vN = h.Sv(vc, i, j + 1, k);
                if (vC > 0 && vN > 0) F = -vC * rho * idy;
                else if (vC < 0 && vN < 0) F = -vN * rho * idy;
                else F = 0;
                if (std::fabs(F) * dy * dy > 2 * mu * sf) {
                    D += -mu * idy2 + min0(F);
                    aN = mu * idy2 + max0(F);
                } else {
                    vm = (vN + vC) * 0.5;
                    Fd = -vm * rho * idy;
                    D += -mu * idy2 + Fd * 0.5;
                    aN = mu * idy2 + Fd * 0.5;
                }
            } else {
                D += -mu * idy2 - (0.25 * rho * idy) * (vC);
            }
        } else {
            D += -mu * idy2 - (0.25 * rho * idy) * (vC);
        }
        if (j - 1 >= 0) {
            if (h.Vm(i, j - 1, k) > -1) {
                double vS = h.Sv(vc, i, j - 1, k);
                if (vC < 0 && vS < 0) F = vC * rho * idy;
                else if (vC > 0 && vS > 0) F = vS * rho * idy;
                else F = 0;
                if (std::fabs(F) * dy * dy > 2 * mu * sf) {
                    D += -mu * idy2 + min0(F);
                    aS = mu * idy2 + max0(F);
                } else {
                    vm = (vS + vC) * 0.5;
                    Fd = vm * rho * idy;
                    D += -mu * idy2 + Fd * 0.5;
                    aS = mu * idy2 + Fd * 0.5;
                }
            } else {
                D += -mu * idy2 + (0.25 * rho * idy) * (vC);
            }
        } else {
            D += -mu * idy2 + (0.25 * rho * idy) * (vC);
        }
        if (nz > 1) {
            if (k + 1 < nz) {
                if (h.Vm(i, j, k + 1) > -1) {
                    wm = (h.Sw(wc, i, j - 1, k + 1) + h.Sw(wc, i, j, k + 1)) * 0.5;
                    F = -wm * rho * idz;
                    if (std::fabs(wm) * rho * dz > 2 * mu * sf) {
                        D += -mu * idz2 + min0(F);
                        aT = mu * idz2 + max0(F);
                    } else {
                        D += -mu * idz2 + F * 0.5;
                        aT = mu * idz2 + F * 0.5;
                    }
                } else {
                    D += -2 * mu * idz2;
                }
            } else {
                D += -2 * mu * idz2;
            }
            if (k - 1 >= 0) {
                if (h.Vm(i, j, k - 1) > -1) {
                    wm = (h.Sw(wc, i, j - 1, k) + h.Sw(wc, i, j, k)) * 0.5;
                    F = wm * rho * idz;
                    if (std::fabs(wm) * rho * dz > 2 * mu * sf) {
                        D += -mu * idz2 + min0(F);
                        aB = mu * idz2 + max0(F);
                    } else {
                        D += -mu * idz2 + F * 0.5;
                        aB = mu * idz2 + F * 0.5;
                    }
                } else {
                    D += -2 * mu * idz2;
                }
            } else {
                D += -2 * mu * idz2;
            }
        }
        D /= h.alpha;
        A.c[SP][(size_t)r] = D;
        A.c[SW][(size_t)r] = aW; A.c[SE][(size_t)r] = aE;
        A.c[SS][(size_t)r] = aS; A.c[SN][(size_t)r] = aN;
        A.c[SB][(size_t)r] = aB; A.c[ST][(size_t)r] = aT;
    }
}

void assemble_mom_z(Handle &h, const std::vector<double> &uc, const std::vector<double> &vc,
                    const std::vector<double> &wc) {
    System &A = h.W;
    const double dx = h.dx, dy = h.dy, dz = h.dz, mu = h.mu, rho = h.rho, sf = h.schemefactor;
    const double idx2 = 1 / (dx * dx), idy2 = 1 / (dy * dy), idz2 = 1 / (dz * dz);
    const double idx = 1 / dx, idy = 1 / dy, idz = 1 / dz;
    const int d0 = h.nx, ny = h.ny, nz = h.nz;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < A.n; ++r) {
        int i, j, k;
        h.ijk(A.cell[(size_t)r], i, j, k);
        double D = 0, F, um, vm, wm, Fd;
        double aW = 0, aE = 0, aS = 0, aN = 0, aB = 0, aT = 0;
        if (i + 1 < d0) {
            if (h.Wm(i + 1, j, k) > -1) {
                um = (h.Su(uc, i + 1, j, k - 1) + h.Su(uc, i + 1, j, k)) * 0.5;
                F = -um * rho * idx;
                if (std::fabs(um) * dx * rho > 2 * mu * sf) {
                    D += -mu * idx2 + min0(F);
                    aE = mu * idx2 + max0(F);
                } else {
                    D += -mu * idx2 + F * 0.5;
                    aE = mu * idx2 + F * 0.5;
                }
            } else {
                D += -2 * mu * idx2;
            }
        } else {
            D += -(0.5 * rho * idx) * (h.Su(uc, i + 1, j, k - 1) + h.Su(uc, i + 1, j, k));
        }
        if (i - 1 >= 0) {
            if (h.Wm(i - 1, j, k) > -1) {
                um = (h.Su(uc, i, j, k - 1) + h.Su(uc, i, j, k)) * 0.5;
                F = um * rho * idx;
                if (std::fabs(um) * dx * rho > 2 * mu * sf) {
                    D += -mu * idx2 + min0(F);
                    aW = mu * idx2 + max0(F);
                } else {
                    D += -mu * idx2 + F * 0.5;
                    aW = mu * idx2 + F * 0.5;
                }
            } else {
                D += -2 * mu * idx2;
            }
        } else {
            D += -mu * idx2 + (0.25 * rho * idx) * (h.Su(uc, i, j, k - 1) + h.Su(uc, i, j, k));
        }
        if (j + 1 < ny) {
            if (h.Wm(i, j + 1, k) > -1) {
                vm = (h.Sv(vc, i, j + 1, k - 1) + h.Sv(vc, i, j + 1, k)) * 0.5;
                F = -vm * rho * idy;
                if (std::fabs(vm) * rho * dy > 2 * mu * sf) {
                    D += -mu * idy2 + min0(F);
                    aN = mu * idy2 + max0(F);
                } else {
                    D += -mu * idy2 + F * 0.5;
                    aN = mu * idy2 + F * 0.5;
                }
            } else {
                D += -2 * mu * idy2;
            }
        } else {
            D += -2 * mu * idy2;
        }
        if (j - 1 >= 0) {
            if (h.Wm(i, j - 1, k) > -1) {
                vm = (h.Sv(vc, i, j, k - 1) + h.Sv(vc, i, j, k)) * 0.5;
                F = vm * rho * idy;
                if (std::fabs(vm) * rho * dy > 2 * mu * sf) {
                    D += -mu * idy2 + min0(F);
                    aS = mu * idy2 + max0(F);
                } else {
                    D += -mu * idy2 + F * 0.5;
                    aS = mu * idy2 + F * 0.5;
                }
            } else {
                D += -2 * mu * idy2;
            }
        } else {
            D += -2 * mu * idy2;
        }
        double wC = h.Sw(wc, i, j, k);
        if (k + 1 < nz) {
            if (h.Wm(i, j, k + 1) > -1) {
                double wT = h.Sw(wc, i, j, k + 1);
                if (wC > 0 && wT > 0) F = -wC * rho * idz;
                else if (wC < 0 && wT < 0) F = -wT * rho * idz;
                else F = 0;
                if (std::fabs(F) * dz * dz > 2 * mu * sf) {
                    D += -mu * idz2 + min0(F);
                    aT = mu * idz2 + max0(F);
                } else {
                    wm = (wC + wT) * 0.5;
                    Fd = -wm * rho * idz;
                    D += -mu * idz2 + Fd * 0.5;
                    aT = mu * idz2 + Fd * 0.5;
                }
            } else {
                D += -mu * idz2 - (0.25 * rho * idz) * (wC);
            }
        } else {
            D += -mu * idz2 - (0.25 * rho * idz) * (wC);
        }
        if (k - 1 >= 0) {
            if (h.Wm(i, j, k - 1) > -1) {
                double wB = h.Sw(wc, i, j, k - 1);
                if (wB < 0 && wC < 0) F = wC * rho * idz;
                else if (wB > 0 && wC > 0) F = wB * rho * idz;
                else F = 0;
                if (std::fabs(F) * dz * dz > 2 * mu * sf) {
                    D += -mu * idz2 + min0(F);
                    aB = mu * idz2 + max0(F);
                } else {
                    wm = (wB + wC) * 0.5;
                    Fd = wm * rho * idz;
                    D += -mu * idz2 + Fd * 0.5;
                    aB = mu * idz2 + Fd * 0.5;
                }
            } else {
                D += -mu * idz2 + (0.25 * rho * idz) * (wC);
            }
        } else {
            D += -mu * idz2 + (0.25 * rho * idz) * (wC);
        }
        D /= h.alpha;
        A.c[SP][(size_t)r] = D;
        A.c[SW][(size_t)r] = aW; A.c[SE][(size_t)r] = aE;
        A.c[SS][(size_t)r] = aS; A.c[SN][(size_t)r] = aN;
        A.c[SB][(size_t)r] = aB; A.c[ST][(size_t)r] = aT;
    }
}

/* AssembleAllMomentum + the Jacobi "factorization", src/NSBase.cxx:853-884 */
void assemble_all_momentum(Handle &h, const std::vector<double> &uc, const std::vector<double> &vc,
                           const std::vector<double> &wc) {
    PhaseTimer phase_timer(0);
    assemble_mom_x(h, uc, vc, wc);
    h.U.compute_invdiag();
    h.U.compute_rowsum();
    assemble_mom_y(h, uc, vc, wc);
    h.V.compute_invdiag();
    h.V.compute_rowsum();
    if (h.nw > 0) {
        assemble_mom_z(h, uc, vc, wc);
        h.W.compute_invdiag();
        h.W.compute_rowsum();
    }
}

/* ---- momentum right-hand sides, src/NSBase.cxx:1445-1546 ---------------- */
void rhs_u(Handle &h) {
    PhaseTimer phase_timer(0);
    System &A = h.U;
    const double idx = 1 / h.dx;
    const int nx = h.nx;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < A.n; ++r) {
        int i, j, k;
        h.ijk(A.cell[(size_t)r], i, j, k);
        double b;
        if (i == 0) b = (h.p[(size_t)h.Pm(i, j, k)] - h.p0) * idx;
        else if (i == nx) b = (h.p1 - h.p[(size_t)h.Pm(i - 1, j, k)]) * idx;
        else b = (h.p[(size_t)h.Pm(i, j, k)] - h.p[(size_t)h.Pm(i - 1, j, k)]) * idx;
        b += h.u[(size_t)r] * A.c[SP][(size_t)r] * (1 - h.alpha);
        A.rhs[(size_t)r] = b;
    }
}
void rhs_v(Handle &h) {
    PhaseTimer phase_timer(0);
    System &A = h.V;
    const double idy = 1 / h.dy;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < A.n; ++r) {
        int i, j, k;
        h.ijk(A.cell[(size_t)r], i, j, k);
        A.rhs[(size_t)r] = (h.p[(size_t)h.Pm(i, j, k)] - h.p[(size_t)h.Pm(i, j - 1, k)]) * idy +
                           h.v[(size_t)r] * A.c[SP][(size_t)r] * (1 - h.alpha);
    }
}
void rhs_w(Handle &h) {
    PhaseTimer phase_timer(0);
    System &A = h.W;
    const double idz = 1 / h.dz;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < A.n; ++r) {
        int i, j, k;
        h.ijk(A.cell[(size_t)r], i, j, k);
        A.rhs[(size_t)r] = (h.p[(size_t)h.Pm(i, j, k)] - h.p[(size_t)h.Pm(i, j, k - 1)]) * idz +
                           h.w[(size_t)r] * A.c[SP][(size_t)r] * (1 - h.alpha);
    }
}

/* ---- pseudo-velocities, src/NSBase.cxx:1548-1755 ------------------------ */
/* order of the off-diagonal products: E, W, N, S, T, B */
void compute_hat(const Handle &h, const System &A, const std::vector<double> &xc, const std::vector<double> &xold,
                 std::vector<double> &hat) {
    PhaseTimer phase_timer(0);
    hat.assign((size_t)A.n, 0.0);
    const int order[6] = {SE, SW, SN, SS, ST, SB};
#pragma omp parallel for schedule(static)
    for (int r = 0; r < A.n; ++r) {
        double t = 0;
        for (int q = 0; q < 6; ++q) {
            int s = order[q];
            int c = A.nb[s - 1][(size_t)r];
            if (c >= 0) t -= A.c[s][(size_t)r] * xc[(size_t)c];
        }
        hat[(size_t)r] = (t) / (A.c[SP][(size_t)r]) + xold[(size_t)r] * (1 - h.alpha);
    }
}

/* ---- pressure systems, src/NSBase.cxx:478-851 --------------------------- */
/* mode 0: AssemblePressure (a_P of the faces), mode 1: pressure correction
 * SIMPLEC (row sums), mode 2: pressure correction SIMPLE (a_P) */
void assemble_pressure_system(Handle &h, int mode, bool relax, const std::vector<double> &uc,
                              const std::vector<double> &vc, const std::vector<double> &wc) {
    PhaseTimer phase_timer(0);
    System &S = h.P;
    const int nx = h.nx, ny = h.ny, nz = h.nz;
    const double dx2 = h.dx * h.dx, dy2 = h.dy * h.dy, dz2 = h.dz * h.dz;
    const double idx = 1 / h.dx, idy = 1 / h.dy, idz = 1 / h.dz;
    const std::vector<double> &au = (mode == 1) ? h.U.rowsum : h.U.c[SP];
    const std::vector<double> &av = (mode == 1) ? h.V.rowsum : h.V.c[SP];
    const std::vector<double> &aw = (mode == 1) ? h.W.rowsum : h.W.c[SP];
#pragma omp parallel for schedule(static)
    for (int r = 0; r < S.n; ++r) {
        int i, j, k;
        h.ijk(S.cell[(size_t)r], i, j, k);
        double D = 0, b = 0;
        double cW = 0, cE = 0, cS = 0, cN = 0, cB = 0, cT = 0;
        int f;
        if (i > 0 && h.Pm(i - 1, j, k) > -1 && (f = h.Um(i, j, k)) > -1) {
            D += 1 / ((au[(size_t)f]) * dx2);
            cW = -1 / ((au[(size_t)f]) * dx2);
            b -= uc[(size_t)f] * idx;
        }
        if (i < nx - 1 && h.Pm(i + 1, j, k) > -1 && (f = h.Um(i + 1, j, k)) > -1) {
            D += 1 / ((au[(size_t)f]) * dx2);
            cE = -1 / ((au[(size_t)f]) * dx2);
            b += uc[(size_t)f] * idx;
        }
        if (j > 0 && h.Pm(i, j - 1, k) > -1 && (f = h.Vm(i, j, k)) > -1) {
            D += 1 / ((av[(size_t)f]) * dy2);
            cS = -1 / ((av[(size_t)f]) * dy2);
            b -= vc[(size_t)f] * idy;
        }
        if (j < ny - 1 && h.Pm(i, j + 1, k) > -1 && (f = h.Vm(i, j + 1, k)) > -1) {
            D += 1 / ((av[(size_t)f]) * dy2);
            cN = -1 / ((av[(size_t)f]) * dy2);
            b += vc[(size_t)f] * idy;
        }
        if (k > 0 && nz > 0 && h.Pm(i, j, k - 1) > -1 && (f = h.Wm(i, j, k)) > -1) {
            D += 1 / ((aw[(size_t)f]) * dz2);
            cB = -1 / ((aw[(size_t)f]) * dz2);
            b -= wc[(size_t)f] * idz;
        }
        if (k < nz - 1 && nz > 0 && h.Pm(i, j, k + 1) > -1 && (f = h.Wm(i, j, k + 1)) > -1) {
            D += 1 / ((aw[(size_t)f]) * dz2);
            cT = -1 / ((aw[(size_t)f]) * dz2);
            b += wc[(size_t)f] * idz;
        }
        if (i == 0 && (f = h.Um(i, j, k)) > -1) {
            D += 1 / ((au[(size_t)f]) * dx2);
            if (mode == 0) b -= uc[(size_t)f] * idx - h.p0 / (au[(size_t)f] * dx2);
            else b -= uc[(size_t)f] * idx;
        }
        if (i == nx - 1 && (f = h.Um(i + 1, j, k)) > -1) {
            D += 1 / ((au[(size_t)f]) * dx2);
            if (mode == 0) b += uc[(size_t)f] * idx + h.p1 / (au[(size_t)f] * dx2);
            else b += uc[(size_t)f] * idx;
        }
        if (mode == 0 && relax) {
            D /= h.beta;
            b += h.p[(size_t)r] * D * (1 - h.beta);
        }
        S.c[SP][(size_t)r] = D;
        S.c[SW][(size_t)r] = cW; S.c[SE][(size_t)r] = cE;
        S.c[SS][(size_t)r] = cS; S.c[SN][(size_t)r] = cN;
        S.c[SB][(size_t)r] = cB; S.c[ST][(size_t)r] = cT;
        S.rhs[(size_t)r] = b;
    }
    S.compute_invdiag();
}

/* ---- velocity corrections, src/NSBase.cxx:2082-2335 --------------------- */
inline double clampdv(double d, double m) {
    if (d < 0 && std::fabs(d) > m) d = -m;
    else if (d > 0 && d > m) d = m;
    return d;
}
/* simplec=1 uses row sums, 0 uses the diagonal */
void correct_velocity_simple(Handle &h, bool simplec, double dvmax) {
    PhaseTimer phase_timer(2);
    const int nx = h.nx, ny = h.ny, nz = h.nz;
    (void)ny;
    const std::vector<double> &au = simplec ? h.U.rowsum : h.U.c[SP];
    const std::vector<double> &av = simplec ? h.V.rowsum : h.V.c[SP];
    const std::vector<double> &aw = simplec ? h.W.rowsum : h.W.c[SP];
    const std::vector<double> &pc = h.pc;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < h.np; ++r) {
        int i, j, k, f, q;
        h.ijk(h.P.cell[(size_t)r], i, j, k);
        double d;
        if (i > 0 && (q = h.Pm(i - 1, j, k)) > -1 && (f = h.Um(i, j, k)) > -1) {
            d = -(pc[(size_t)q] - pc[(size_t)r]) / ((au[(size_t)f]) * h.dx);
            h.u[(size_t)f] = h.u[(size_t)f] + clampdv(d, dvmax);
        }
        if (j > 0 && (q = h.Pm(i, j - 1, k)) > -1 && (f = h.Vm(i, j, k)) > -1) {
            d = -(pc[(size_t)q] - pc[(size_t)r]) / ((av[(size_t)f]) * h.dy);
            h.v[(size_t)f] = h.v[(size_t)f] + clampdv(d, dvmax);
        }
        if (k > 0 && (q = h.Pm(i, j, k - 1)) > -1 && (f = h.Wm(i, j, k)) > -1) {
            d = -(pc[(size_t)q] - pc[(size_t)r]) / ((aw[(size_t)f]) * h.dz);
            h.w[(size_t)f] = h.w[(size_t)f] + clampdv(d, dvmax);
        }
        if (i == 0 && (f = h.Um(i, j, k)) > -1) {
            d = (pc[(size_t)r]) / ((au[(size_t)f]) * h.dx);
            h.u[(size_t)f] = h.u[(size_t)f] + clampdv(d, dvmax);
        }
        if (i == nx - 1 && (f = h.Um(i + 1, j, k)) > -1) {
            d = -(pc[(size_t)r]) / ((au[(size_t)f]) * h.dx);
            h.u[(size_t)f] = h.u[(size_t)f] + clampdv(d, dvmax);
        }
        (void)nz;
    }
}

void correct_velocity_simpler(Handle &h, const std::vector<double> &pp, std::vector<double> &uc,
                              std::vector<double> &vc, std::vector<double> &wc, const std::vector<double> &uh,
                              const std::vector<double> &vh, const std::vector<double> &wh, double p_0,
                              double p_1) {
    PhaseTimer phase_timer(2);
    const int nx = h.nx;
    const std::vector<double> &au = h.U.c[SP], &av = h.V.c[SP], &aw = h.W.c[SP];
#pragma omp parallel for schedule(static)
    for (int r = 0; r < h.np; ++r) {
        int i, j, k, f, q;
        h.ijk(h.P.cell[(size_t)r], i, j, k);
        if (i > 0 && (q = h.Pm(i - 1, j, k)) > -1 && (f = h.Um(i, j, k)) > -1)
            uc[(size_t)f] = uh[(size_t)f] - (pp[(size_t)q] - pp[(size_t)r]) / (au[(size_t)f] * h.dx);
        if (j > 0 && (q = h.Pm(i, j - 1, k)) > -1 && (f = h.Vm(i, j, k)) > -1)
            vc[(size_t)f] = vh[(size_t)f] - (pp[(size_t)q] - pp[(size_t)r]) / (av[(size_t)f] * h.dy);
        if (k > 0 && (q = h.Pm(i, j, k - 1)) > -1 && (f = h.Wm(i, j, k)) > -1)
            wc[(size_t)f] = wh[(size_t)f] - (pp[(size_t)q] - pp[(size_t)r]) / (aw[(size_t)f] * h.dz);
        if (i == 0 && (f = h.Um(i, j, k)) > -1)
            uc[(size_t)f] = uh[(size_t)f] - (p_0 - pp[(size_t)r]) / (au[(size_t)f] * h.dx);
        if (i == nx - 1 && (f = h.Um(i + 1, j, k)) > -1)
            uc[(size_t)f] = uh[(size_t)f] - (pp[(size_t)r] - p_1) / (au[(size_t)f] * h.dx);
    }
}

/* ---- linear solves: src/NSBase.cxx:1773-1884, 2337-2423 ----------------- */
void log_solve(Handle &h, const char *comp, const SolveOut &o) {
    h.info.s("Solving for component ");
    h.info.s(comp);
    h.info.s(" in ");
    h.info.i(o.iters);
    h.info.s(" iterations (status ");
    h.info.i(o.info);
    h.info.s(")");
    h.info.nl();
}

void velocity_component(Handle &h, System &A, std::vector<double> &x, void (*rhs)(Handle &), bool limit,
                        double dvmax, SolveOut &so, const char *comp) {
    rhs(h);
    std::vector<double> temp = x;
    so = bicgstab(A, A.rhs, x, h.prm.vsolvertol, h.prm.maxitsolver, &h.res.krylov_rows);
    h.res.krylov_iterations += so.work;
    if (so.iters == 0 || so.info != 0) x = temp;
    if (limit) {
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)x.size(); ++i) {
            double d = x[(size_t)i] - temp[(size_t)i];
            if (std::fabs(d) > dvmax) {
                if (d > 0) x[(size_t)i] = temp[(size_t)i] + dvmax;
                else if (d < 0) x[(size_t)i] = temp[(size_t)i] - dvmax;
            }
        }
    }
    log_solve(h, comp, so);
}

void compute_velocity_field(Handle &h, bool limit, double dvmax) {
    velocity_component(h, h.U, h.u, rhs_u, limit, dvmax, h.su, "u");
    velocity_component(h, h.V, h.v, rhs_v, limit, dvmax, h.sv, "v");
    if (h.nw > 0) velocity_component(h, h.W, h.w, rhs_w, limit, dvmax, h.sw, "w");
}

void log_pressure_status(Handle &h, const SolveOut &o) {
    if (o.info == NS3D_SUCCESS) {
        h.info.i(o.iters);
        h.info.s(" iterations (status ");
        h.info.i(o.info);
        h.info.s(")");
        h.info.nl();
    } else {
        if (o.info == NS3D_NUMERICAL_ISSUE) { h.info.s("Numerical Issue (iterations:"); h.info.i(o.iters); h.info.s("). "); }
        else if (o.info == NS3D_NO_CONVERGENCE) { h.info.s("No convergence (iterations:"); h.info.i(o.iters); h.info.s("). "); }
        else if (o.info == NS3D_INVALID_INPUT) { h.info.s("Invalid input (iterations:"); h.info.i(o.iters); h.info.s("). "); }
        h.info.s("Residual: ");
        int pr = h.info.prec;
        h.info.d(o.error);
        h.info.prec = pr;
        h.info.nl();
    }
}

void compute_pressure_correction(Handle &h) {
    h.info.s("Solving for pressure correction : ");
    h.sp = bicgstab(h.P, h.P.rhs, h.pc, h.prm.pcsolvertol, h.prm.maxitsolver, &h.res.krylov_rows);
    h.res.krylov_iterations += h.sp.work;
    log_pressure_status(h, h.sp);
}

void compute_pressure_field(Handle &h) {
    double tol = h.prm.psolvertol;
    h.info.s("Solving for pressure in : ");
    std::vector<double> ptemp = h.p;
    h.sp = bicgstab(h.P, h.P.rhs, ptemp, tol, h.prm.maxitsolver, &h.res.krylov_rows);
    h.res.krylov_iterations += h.sp.work;
    while (h.sp.iters == 0 && h.sp.info == NS3D_SUCCESS && tol > 1e-15) {
        tol *= 0.1;
        h.sp = bicgstab(h.P, h.P.rhs, ptemp, tol, h.prm.maxitsolver, &h.res.krylov_rows);
        h.res.krylov_iterations += h.sp.work;
    }
    if (h.sp.iters > 0) h.p = ptemp;
    log_pressure_status(h, h.sp);
}

/* CorrectPressureField, src/NSBase.cxx:2367-2380 */
void correct_pressure_field(Handle &h) {
    PhaseTimer phase_timer(2);
    double mx = -HUGE_VAL, mn = HUGE_VAL;
    for (int r = 0; r < h.np; ++r) {
        double x = h.pc[(size_t)r];
        mx = (x > mx) ? x : mx;
        mn = (x < mn) ? x : mn;
    }
    double sq = det_dot(h.pc, h.pc, h.np);
    h.pcmax = h.beta * mx;
    h.pcmin = h.beta * mn;
    h.pcnorm = h.beta * std::sqrt(sq);
    h.info.s("Correction de pression maximale et minimale: ");
    h.info.d(h.pcmax);
    h.info.s(", ");
    h.info.d(h.pcmin);
    h.info.nl();
    h.info.s("Norme de la correction de pression : ");
    h.info.d(h.pcnorm);
    h.info.nl();
#pragma omp parallel for schedule(static)
    for (int r = 0; r < h.np; ++r) h.p[(size_t)r] = h.p[(size_t)r] + h.beta * h.pc[(size_t)r];
}

/* ---- diagnostics: src/NSBase.cxx:1886-2080 ------------------------------ */
void compute_permeability(Handle &h, double &Q, double &v_moy, double &K) {
    PhaseTimer phase_timer(3);
    const int nx = h.nx, ny = h.ny, nz = h.nz, b = h.border;
    const double sx = h.dy * h.dz;
    const long plane = (long)ny * nz;
    if (b <= 0) {
        const int iu = nx;  // uindex.shape()(0)-1
        v_moy = det_sum(plane, [&](long q, double acc) {
            int r = h.uindex[(size_t)((long)iu * plane + q)];
            return r > -1 ? acc + h.u[(size_t)r] : acc;
        });
        h.p_inlet = h.p0;
        h.p_outlet = h.p1;
    } else {
        const int iu = nx + 1 - b;  // uindex.shape()(0)-border
        v_moy = det_sum(plane, [&](long q, double acc) {
            int r = h.uindex[(size_t)((long)iu * plane + q)];
            return r > -1 ? acc + h.u[(size_t)r] : acc;
        });
        const int io = nx - b, ii = b - 1;
        double so = det_sum(plane, [&](long q, double acc) {
            int r = h.pindex[(size_t)((long)io * plane + q)];
            return r > -1 ? acc + h.p[(size_t)r] : acc;
        });
        double si = det_sum(plane, [&](long q, double acc) {
            int r = h.pindex[(size_t)((long)ii * plane + q)];
            return r > -1 ? acc + h.p[(size_t)r] : acc;
        });
        int cnt_o = 0, cnt_i = 0;
        for (long q = 0; q < plane; ++q) {
            cnt_o += h.pindex[(size_t)((long)io * plane + q)] > -1;
            cnt_i += h.pindex[(size_t)((long)ii * plane + q)] > -1;
        }
        h.p_inlet = si;
        h.p_outlet = so;
        if (cnt_i > 0) h.p_inlet /= cnt_i;
        if (cnt_o > 0) h.p_outlet /= cnt_o;
    }
    Q = v_moy * sx;
    v_moy /= (ny * nz);
    if (std::fabs(h.p_inlet - h.p_outlet) > 0.0)
        K = v_moy * h.mu * h.dx * (nx - 2 * b) / (h.p_inlet - h.p_outlet);
    else
        K = 0.0;
}

void compute_div(Handle &h, double &MaxDeltaV, double &normdiv, double &velocityNorm, double &maxdiv) {
    PhaseTimer phase_timer(3);
    const int nx = h.nx, ny = h.ny, nz = h.nz;
    const double idx = 1 / h.dx, idy = 1 / h.dy, idz = 1 / h.dz;
    std::vector<double> dv((size_t)h.np), vel((size_t)h.np), dV((size_t)h.np);
#pragma omp parallel for schedule(static)
    for (int r = 0; r < h.np; ++r) {
        int i, j, k, f;
        h.ijk(h.P.cell[(size_t)r], i, j, k);
        double div = 0, uu = 0, vv = 0, ww = 0, DV = 0;
        if (i > 0 && h.Pm(i - 1, j, k) > -1 && (f = h.Um(i, j, k)) > -1) {
            div += -h.u[(size_t)f] * idx; DV += -h.u[(size_t)f]; uu += h.u[(size_t)f] * 0.5;
        }
        if (i < nx - 1 && h.Pm(i + 1, j, k) > -1 && (f = h.Um(i + 1, j, k)) > -1) {
            div += h.u[(size_t)f] * idx; DV += h.u[(size_t)f]; uu += h.u[(size_t)f] * 0.5;
        }
        if (j > 0 && h.Pm(i, j - 1, k) > -1 && (f = h.Vm(i, j, k)) > -1) {
            div += -h.v[(size_t)f] * idy; DV += -h.v[(size_t)f]; vv += h.v[(size_t)f] * 0.5;
        }
        if (j < ny - 1 && h.Pm(i, j + 1, k) > -1 && (f = h.Vm(i, j + 1, k)) > -1) {
            div += h.v[(size_t)f] * idy; DV += h.v[(size_t)f]; vv += h.v[(size_t)f] * 0.5;
        }
        if (k > 0 && nz > 0 && h.Pm(i, j, k - 1) > -1 && (f = h.Wm(i, j, k)) > -1) {
            div += -h.w[(size_t)f] * idz; DV += -h.w[(size_t)f]; ww += h.w[(size_t)f] * 0.5;
        }
        if (k < nz - 1 && nz > 0 && h.Pm(i, j, k + 1) > -1 && (f = h.Wm(i, j, k + 1)) > -1) {
            div += h.w[(size_t)f] * idz; DV += h.w[(size_t)f]; ww += h.w[(size_t)f] * 0.5;
        }
        if (i == 0 && (f = h.Um(i, j, k)) > -1) {
            div += -h.u[(size_t)f] * idx; DV += -h.u[(size_t)f]; uu += h.u[(size_t)f] * 0.5;
        }
        if (i == nx - 1 && (f = h.Um(i + 1, j, k)) > -1) {
            div += h.u[(size_t)f] * idx; DV += h.u[(size_t)f]; uu += h.u[(size_t)f] * 0.5;
        }
        dV[(size_t)r] = std::fabs(DV);
        dv[(size_t)r] = std::fabs(div);
        vel[(size_t)r] = std::sqrt(uu * uu + vv * vv + ww * ww);
    }
    // maxima start at 0 (the reference leaves its max accumulator uninitialised)
    double md = 0, mdv = 0;
    for (int r = 0; r < h.np; ++r) {
        md = (dv[(size_t)r] > md) ? dv[(size_t)r] : md;
        mdv = (dV[(size_t)r] > mdv) ? dV[(size_t)r] : mdv;
    }
    double tempdiv = det_sum(h.np, [&](long r, double acc) { return std::fma(dv[(size_t)r], dv[(size_t)r], acc); });
    double tempvel = det_sum(h.np, [&](long r, double acc) { return acc + vel[(size_t)r]; });
    normdiv = std::sqrt(tempdiv);
    velocityNorm = tempvel / h.np;
    maxdiv = md;
    MaxDeltaV = mdv;
}

/* ---- relaxation / convergence control, src/NSBase.cxx:196-328 ----------- */
void relax_control(Handle &h, bool beta_cst) {
    const size_t size = 30;
    bool isDecreasing = false;
    if (h.RMR > h.old_RMR * h.maxconvdelta) {
        h.alpha = std::max(h.min_alpha, h.alpha - h.relax);
        if (!beta_cst) h.beta = std::max(h.min_beta, h.beta - h.relax);
        h.old_RMR *= 1.1;
        h.info.s("Relative Mass Residual increases too much -> new relaxation parameter alpha, beta: ");
        h.info.d(h.alpha);
        h.info.s(", ");
        h.info.d(h.beta);
        h.info.nl();
        if (!h.avgRMR.empty()) h.avgRMR.pop_front();
    }
    if (!h.avgRMR.empty()) isDecreasing = h.avgRMR.back() > h.RMR;
    h.avgRMR.push_back(h.RMR);
    if (h.avgRMR.size() > size) {
        h.avgRMR.pop_front();
        int i = 0, n1 = 0, n2 = 0;
        double avg1 = 0, avg2 = 0;
        for (double x : h.avgRMR) {
            i += 1;
            if (i < h.avgRMR.size() * 0.5) { avg1 += x; n1 += 1; }
            else if (i >= h.avgRMR.size() * 0.5) { avg2 += x; n2 += 1; }
        }
        avg1 /= n1;
        avg2 /= n2;
        double delta = (avg2 - avg1) / std::max(avg1, avg2);
        if (delta <= 0 && std::fabs(delta) < h.deltaRMR && isDecreasing == false) {
            for (int c = 0; c < 15 && !h.avgRMR.empty(); ++c) h.avgRMR.pop_front();
            h.alpha = std::min(h.alpha0, h.alpha - h.relax * 0.25);
            if (!beta_cst) h.beta = std::max(h.min_beta, h.beta - h.relax * 0.25);
            h.info.s("Simulation is oscillating -> new relaxation parameter alpha, beta: ");
            h.info.d(h.alpha);
            h.info.s(", ");
            h.info.d(h.beta);
            h.info.nl();
        } else if (delta > 0 && isDecreasing == false) {
            for (int c = 0; c < 15 && !h.avgRMR.empty(); ++c) h.avgRMR.pop_front();
            h.alpha = std::max(h.min_alpha, h.alpha - h.relax);
            if (!beta_cst) h.beta = std::max(h.min_beta, h.beta - h.relax);
            h.info.s("Simulation is diverging -> new relaxation parameter alpha, beta: ");
            h.info.d(h.alpha);
            h.info.s(", ");
            h.info.d(h.beta);
            h.info.nl();
        }
    }
}

bool check_convergence(Handle &h, double res, double tol) {
    if (res < tol) return true;
    if (h.su.iters == 0 && h.sv.iters == 0 && (h.nw == 0 || h.sw.iters == 0) && h.sp.iters == 0) return true;
    return false;
}

/* ---- outer loops --------------------------------------------------------- */
const char *kResHeader =
    "iteration, Q (m³/s), <u_out> (m/s), Max Rel Mass Res., K (m²), gradP (Pa/m), ||Div_u||, "
    "Lref*(max DIV)/<u_out>, <||u||>, max DIV, it_u,it_v,it_w,it_pc";

struct Iter {
    double Q = 0, v_moy = 0, K = 0, normdiv = 0, reldiv = 0, velocityNorm = 0, maxdiv = 0, MaxDeltaV = 0;
};

void res_row(Handle &h, int it, const Iter &s) {
    Log &L = h.resl;
    if (!L.f) return;
    L.i(it); L.s(","); L.d(s.Q); L.s(","); L.d(s.v_moy); L.s(","); L.d(h.RMR); L.s(","); L.d(s.K); L.s(",");
    L.d((h.p_inlet - h.p_outlet) / (h.dx * (h.nx - 2 * h.border)));
    L.s(","); L.d(s.normdiv); L.s(","); L.d(s.reldiv); L.s(","); L.d(s.velocityNorm); L.s(", "); L.d(s.maxdiv);
    L.s(", ");
    L.i(h.su.valid ? h.su.iters : 0); L.s(",");
    L.i(h.sv.valid ? h.sv.iters : 0); L.s(",");
    L.i(h.sw.valid ? h.sw.iters : 0); L.s(",");
    L.i(h.sp.valid ? h.sp.iters : 0);
    L.nl();
}

void info_K(Handle &h, const char *what, double K) {
    h.info.s(what);
    h.info.d(K);
    h.info.nl();
}

void diagnostics(Handle &h, Iter &s) {
    compute_permeability(h, s.Q, s.v_moy, s.K);
    compute_div(h, s.MaxDeltaV, s.normdiv, s.velocityNorm, s.maxdiv);
    h.RMR = s.MaxDeltaV / std::fabs(s.v_moy);
    s.reldiv = (h.nx * h.dx + h.ny * h.dy + h.nz * h.dz) * s.maxdiv / (3 * s.v_moy);
    info_K(h, "Permeability K (m²): ", s.K);
}

void old_rmr_update(Handle &h, int it) {
    if (it > 1) {
        if (h.RMR < h.old_RMR) h.old_RMR = h.RMR;
    } else {
        h.old_RMR = h.RMR;
    }
}

void fields_to_image_log(Handle &h, const std::string &file) {
    const char *pre[5] = {"Vx-", "Vy-", "Vz-", "V-", "P-"};
    for (auto p : pre) {
        h.info.s("Writing ");
        h.info.s(p);
        h.info.i(h.prm.direction);
        h.info.s("-");
        h.info.s(file.c_str());
        h.info.nl();
    }
}

void save_snapshot(Handle &h, int it, int &savecounter) {
    if (it % h.prm.save_step == 0 && it > 0) {
        savecounter += 1;
        if (savecounter > 3) savecounter = 1;
        fields_to_image_log(h, h.stem + "-SAVE-" + std::to_string(savecounter) + ".vti");
    }
}

void init_fields_and_header(Handle &h, const char *name, const char *maxname) {
    h.info.s("Initializing ");
    h.info.s(name);
    h.info.s(" algorithm");
    h.info.nl();
    // Initpvector's log lines (the fields themselves are set beforehand)
    h.info.s("p0, p1 (Pa)= "); h.info.d(h.p0); h.info.s(","); h.info.d(h.p1); h.info.nl();
    h.info.s("Pressure gradient (Pa/m)= "); h.info.d((h.p0 - h.p1) / (h.dx * h.nx)); h.info.nl();
    h.info.s("inlet/outlet area (m²)= "); h.info.d(h.dy * h.dz * h.ny * h.nz); h.info.nl();
    h.info.s(maxname); h.info.i(h.prm.maxitSIMPLE); h.info.nl();
    if (h.resl.f) { h.resl.s(kResHeader); h.resl.nl(); }
}

void finish(Handle &h, const char *name, int it, const Iter &s, std::chrono::steady_clock::time_point t0,
            time_t start) {
    h.info.s("Norm of the velocity field divergence: "); h.info.d(s.normdiv); h.info.nl();
    h.info.s("Relative divergence of the velocity field: "); h.info.d(s.reldiv); h.info.nl();
    fields_to_image_log(h, h.stem + ".vti");
    time_t end = time(0);
    h.info.s(name); h.info.s(" terminated in "); h.info.i(it); h.info.s(" iteration and ");
    h.info.d(difftime(end, start)); h.info.s(" seconds"); h.info.nl();
    ns3d_result &R = h.res;
    R.K = s.K; R.Q = s.Q; R.v_moy = s.v_moy; R.RMR = h.RMR;
    R.normdiv = s.normdiv; R.reldiv = s.reldiv; R.velocityNorm = s.velocityNorm; R.maxdiv = s.maxdiv;
    R.MaxDeltaV = s.MaxDeltaV; R.p_inlet = h.p_inlet; R.p_outlet = h.p_outlet; R.p0 = h.p0; R.p1 = h.p1;
    R.alpha = h.alpha; R.beta = h.beta; R.pcmax = h.pcmax; R.pcmin = h.pcmin; R.pcnorm = h.pcnorm;
    R.iterations = it;
    R.it_u = h.su.valid ? (int)h.su.iters : 0;
    R.it_v = h.sv.valid ? (int)h.sv.iters : 0;
    R.it_w = h.sw.valid ? (int)h.sw.iters : 0;
    R.it_p = h.sp.valid ? (int)h.sp.iters : 0;
    R.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void initial_velocity(Handle &h, Iter &s) {
    assemble_all_momentum(h, h.u, h.v, h.w);
    compute_velocity_field(h, false, 0);
    compute_permeability(h, s.Q, s.v_moy, s.K);
    info_K(h, "Initial Permeability K (m²): ", s.K);
}

/* SIMPLECSOLVER::Solve, src/SIMPLEC.cxx:73-232 */
void run_simplec(Handle &h) {
    auto t0 = std::chrono::steady_clock::now();
    time_t start = time(0);
    Iter s;
    int savecounter = 0, it;
    init_fields_and_header(h, "SIMPLEC", "Max number of SIMPLE iterations: ");
    h.alpha = h.alpha0;
    initial_velocity(h, s);
    for (it = 0; it < h.prm.maxitSIMPLE; ++it) {
        h.info.s("Iteration "); h.info.i(it); h.info.s("  ------------"); h.info.nl();
        if (it > 0) {
            assemble_all_momentum(h, h.u, h.v, h.w);
            compute_velocity_field(h, true, s.v_moy * std::min(1., h.alpha * 1.5));
        }
        diagnostics(h, s);
        old_rmr_update(h, it);
        res_row(h, it, s);
        if (it > 1 && check_convergence(h, h.RMR, h.prm.simpletol)) {
            info_K(h, "Permeability K (m²): ", s.K);
            h.res.converged = 1;
            break;
        }
        assemble_pressure_system(h, 1, false, h.u, h.v, h.w);
        compute_pressure_correction(h);
        correct_velocity_simple(h, true, s.v_moy * h.alpha);
        correct_pressure_field(h);
        Iter after = s;
        compute_div(h, after.MaxDeltaV, after.normdiv, after.velocityNorm, after.maxdiv);
        s.MaxDeltaV = after.MaxDeltaV; s.normdiv = after.normdiv; s.velocityNorm = after.velocityNorm; s.maxdiv = after.maxdiv;
        save_snapshot(h, it, savecounter);
        relax_control(h, true);
    }
    finish(h, "SIMPLEC", it, s, t0, start);
}

void pressure_step(Handle &h, bool relax, std::vector<double> &uc, std::vector<double> &vc, std::vector<double> &wc,
                   const std::vector<double> &uold, const std::vector<double> &vold, const std::vector<double> &wold,
                   std::vector<double> &ut, std::vector<double> &vt, std::vector<double> &wt,
                   std::vector<double> &uh, std::vector<double> &vh, std::vector<double> &wh) {
    // Compute_{u,v,w}_hat(hat, A, xc, xold); AssemblePressure; ComputePressureField;
    // CorrectVelocityFieldSIMPLER(p, ut, vt, wt, hats, p0, p1)
    compute_hat(h, h.U, uc, uold, uh);
    compute_hat(h, h.V, vc, vold, vh);
    compute_hat(h, h.W, wc, wold, wh);
    assemble_pressure_system(h, 0, relax, uh, vh, wh);
    compute_pressure_field(h);
    correct_velocity_simpler(h, h.p, ut, vt, wt, uh, vh, wh, h.p0, h.p1);
}

/* SIMPLER / SIMPLERR / IDEAL drivers, src/SIMPLER.cxx:75-270,
 * src/SIMPLERR.cxx:75-280, src/IDEAL.cxx:75-281 */
void run_simpler_family(Handle &h, int method) {
    auto t0 = std::chrono::steady_clock::now();
    time_t start = time(0);
    Iter s;
    int savecounter = 0, it;
    const char *name = method == NS3D_SIMPLER ? "SIMPLER" : method == NS3D_SIMPLERR ? "SIMPLER-R" : "IDEAL";
    const char *maxname = method == NS3D_SIMPLER    ? "Max number of SIMPLE iterations: "
                          : method == NS3D_SIMPLERR ? "Max number of SIMPLE-R iterations: "
                                                    : "Max number of IDEAL iterations: ";
    std::vector<double> uh((size_t)h.nu, 0.0), vh((size_t)h.nv, 0.0), wh((size_t)h.nw, 0.0);
    std::vector<double> ut((size_t)h.nu, 0.0), vt((size_t)h.nv, 0.0), wt((size_t)h.nw, 0.0);
    init_fields_and_header(h, name, maxname);
    initial_velocity(h, s);
    h.alpha = h.alpha0;
    const bool relax = true;
    for (it = 0; it < h.prm.maxitSIMPLE; ++it) {
        h.info.s("Iteration "); h.info.i(it); h.info.s("  ------------"); h.info.nl();
        assemble_all_momentum(h, h.u, h.v, h.w);
        ut = h.u; vt = h.v; wt = h.w;
        for (int sub = 0; sub < h.prm.N1; ++sub)
            pressure_step(h, relax, ut, vt, wt, h.u, h.v, h.w, ut, vt, wt, uh, vh, wh);
        compute_velocity_field(h, true, s.v_moy * std::min(1., h.alpha * 1.5));
        diagnostics(h, s);
        old_rmr_update(h, it);
        if (method == NS3D_SIMPLER) res_row(h, it, s);
        if (it > 1 && check_convergence(h, h.RMR, h.prm.simpletol)) {
            info_K(h, "Permeability K (m²): ", s.K);
            h.res.converged = 1;
            break;
        }
        Iter after = s;
        if (method == NS3D_SIMPLER || method == NS3D_SIMPLERR) {
            assemble_pressure_system(h, 2, false, h.u, h.v, h.w);
            compute_pressure_correction(h);
            correct_velocity_simple(h, false, s.v_moy * 100);
            if (method == NS3D_SIMPLERR) {
                compute_hat(h, h.U, h.u, h.u, uh);
                compute_hat(h, h.V, h.v, h.v, vh);
                compute_hat(h, h.W, h.w, h.w, wh);
                assemble_pressure_system(h, 0, relax, uh, vh, wh);
                compute_pressure_field(h);
            }
        } else {  // IDEAL step 3
            ut = h.u; vt = h.v; wt = h.w;
            for (int sub = 0; sub < h.prm.N2; ++sub)
                pressure_step(h, false, h.u, h.v, h.w, ut, vt, wt, h.u, h.v, h.w, uh, vh, wh);
        }
        compute_div(h, after.MaxDeltaV, after.normdiv, after.velocityNorm, after.maxdiv);
        s.MaxDeltaV = after.MaxDeltaV; s.normdiv = after.normdiv; s.velocityNorm = after.velocityNorm; s.maxdiv = after.maxdiv;
        if (method == NS3D_SIMPLERR) {
            res_row(h, it, s);
            relax_control(h, false);
            save_snapshot(h, it, savecounter);
        } else {
            save_snapshot(h, it, savecounter);
            relax_control(h, true);
        }
    }
    finish(h, name, it, s, t0, start);
}

void default_fields(Handle &h) {
    h.p.assign((size_t)h.np, 0.0);
    h.u.assign((size_t)h.nu, 0.0);
    h.v.assign((size_t)h.nv, 0.0);
    h.w.assign((size_t)h.nw, 0.0);
    h.pc.assign((size_t)h.np, 0.0);
    // Initpvector default profile, src/NSBase.cxx:2671-2681
    for (int r = 0; r < h.np; ++r) {
        int i, j, k;
        h.ijk(h.P.cell[(size_t)r], i, j, k);
        h.p[(size_t)r] = (h.p1 - h.p0) * ((double)i + 1.0) / ((double)h.nx) + h.p0;
    }
    h.fields_ready = true;
}

}  // namespace

struct ns3d_handle {
    Handle h;
};

extern "C" {

NS3D_API int ns3d_abi_version(void) { return NS3D_ABI_VERSION; }
NS3D_API const char *ns3d_backend_name(void) { return "oracle"; }
NS3D_API const char *ns3d_last_error(void) { return g_err.c_str(); }

NS3D_API void ns3d_params_default(ns3d_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->dx = 1.0; p->dy = -1.0; p->dz = -1.0;
    p->mu = 1e-3; p->rho = 1e3; p->p0 = 1e5; p->gradp = 1e2;
    p->alpha = 0.8; p->beta = 1.0;
    p->vsolvertol = 1e-5; p->psolvertol = 1e-6; p->pcsolvertol = 1e-3;
    p->simpletol = 1e-4; p->deltaRMR = 1e-4;
    p->maxitsolver = 1000; p->maxitSIMPLE = 500; p->N1 = 2; p->N2 = 2; p->save_step = 20;
    p->porevalue = 0; p->direction = 1; p->border = 0;
    p->method = NS3D_SIMPLEC; p->precision = NS3D_FP64;
}

NS3D_API int ns3d_open(const ns3d_params *params, const uint8_t *raw, int32_t nx, int32_t ny, int32_t nz,
                       ns3d_handle **out) {
    if (!params || !raw || !out) return fail(NS3D_ERR_ARG, "ns3d_open: NULL argument");
    read_arith_mode();
    if (nx <= 0 || ny <= 0 || nz <= 0) return fail(NS3D_ERR_ARG, "ns3d_open: bad image size");
    if ((long)nx * ny * nz > 0x7fffffffL) return fail(NS3D_ERR_ARG, "ns3d_open: image too large");
    if (params->direction < 1 || params->direction > 3) return fail(NS3D_ERR_ARG, "ns3d_open: direction must be 1, 2 or 3");
    if (params->dx <= 0 || params->mu <= 0 || params->rho <= 0 || params->maxitsolver <= 0 || params->maxitSIMPLE <= 0 ||
        params->save_step <= 0 || params->border < 0)
        return fail(NS3D_ERR_ARG, "ns3d_open: invalid parameter");
    ns3d_handle *H = new ns3d_handle();
    Handle &h = H->h;
    h.prm = *params;
    if (h.prm.dy <= 0) h.prm.dy = h.prm.dx;
    if (h.prm.dz <= 0) h.prm.dz = h.prm.dx;
    if (h.prm.porevalue != 0 && h.prm.porevalue != 1) h.prm.porevalue = 0;
    build_geometry(h, raw, nx, ny, nz);
    build_systems(h);
    h.dx = h.prm.dx; h.dy = h.prm.dy; h.dz = h.prm.dz; h.mu = h.prm.mu; h.rho = h.prm.rho;
    h.p0 = h.prm.p0; h.gradp = h.prm.gradp; h.border = h.prm.border; h.deltaRMR = h.prm.deltaRMR;
    // constructor constants, src/NSBase.cxx:155-179
    h.p1 = -h.gradp * (h.dx * h.nx) + h.p0;
    if (h.p1 < 0) { h.p0 -= h.p1; h.p1 = 0; }
    h.schemefactor = 0; h.min_alpha = 0.001; h.min_beta = 0.001; h.relax = 0.05;
    h.speedup = h.relax * 0.5; h.maxconvdelta = 2.5;
    h.alpha = h.alpha0 = h.prm.alpha;
    h.beta = h.beta0 = h.prm.beta;
    std::memset(&h.res, 0, sizeof h.res);
    default_fields(h);
    *out = H;
    return NS3D_OK;
}

NS3D_API int ns3d_get_sizes(const ns3d_handle *H, ns3d_sizes *s) {
    if (!H || !s) return fail(NS3D_ERR_ARG, "NULL argument");
    const Handle &h = H->h;
    s->nx = h.nx; s->ny = h.ny; s->nz = h.nz; s->np = h.np; s->nu = h.nu; s->nv = h.nv; s->nw = h.nw; s->reserved = 0;
    return NS3D_OK;
}

NS3D_API int ns3d_get_index_arrays(ns3d_handle *H, int32_t *pi, int32_t *ui, int32_t *vi, int32_t *wi) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    if (pi) std::memcpy(pi, h.pindex.data(), h.pindex.size() * 4);
    if (ui) std::memcpy(ui, h.uindex.data(), h.uindex.size() * 4);
    if (vi) std::memcpy(vi, h.vindex.data(), h.vindex.size() * 4);
    if (wi) std::memcpy(wi, h.windex.data(), h.windex.size() * 4);
    return NS3D_OK;
}

NS3D_API int ns3d_set_initial_fields(ns3d_handle *H, const double *pimg, const double *uimg, const double *vimg,
                                     const double *wimg) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    default_fields(h);
    if (pimg)
        for (size_t c = 0; c < h.pindex.size(); ++c)
            if (h.pindex[c] != -1) h.p[(size_t)h.pindex[c]] = pimg[c];
    if (uimg)
        for (size_t c = 0; c < h.uindex.size(); ++c)
            if (h.uindex[c] != -1) h.u[(size_t)h.uindex[c]] = uimg[c];
    if (vimg)
        for (size_t c = 0; c < h.vindex.size(); ++c)
            if (h.vindex[c] != -1) h.v[(size_t)h.vindex[c]] = vimg[c];
    if (wimg)
        for (size_t c = 0; c < h.windex.size(); ++c)
            if (h.windex[c] != -1) h.w[(size_t)h.windex[c]] = wimg[c];
    return NS3D_OK;
}

NS3D_API int ns3d_get_fields(ns3d_handle *H, double *p, double *u, double *v, double *w) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    if (p) std::memcpy(p, h.p.data(), h.p.size() * 8);
    if (u) std::memcpy(u, h.u.data(), h.u.size() * 8);
    if (v) std::memcpy(v, h.v.data(), h.v.size() * 8);
    if (w) std::memcpy(w, h.w.data(), h.w.size() * 8);
    return NS3D_OK;
}

NS3D_API int ns3d_set_fields(ns3d_handle *H, const double *p, const double *u, const double *v, const double *w) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    if (p) std::memcpy(h.p.data(), p, h.p.size() * 8);
    if (u) std::memcpy(h.u.data(), u, h.u.size() * 8);
    if (v) std::memcpy(h.v.data(), v, h.v.size() * 8);
    if (w) std::memcpy(h.w.data(), w, h.w.size() * 8);
    return NS3D_OK;
}

NS3D_API int ns3d_get_field_images(ns3d_handle *H, double *pimg, double *uimg, double *vimg, double *wimg,
                                   double *vavg) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    const int nx = h.nx, ny = h.ny, nz = h.nz;
    const size_t N = (size_t)nx * ny * nz;
    if (pimg) for (size_t c = 0; c < N; ++c) pimg[c] = h.pindex[c] > -1 ? h.p[(size_t)h.pindex[c]] : 0.0;
    if (uimg) for (size_t c = 0; c < h.uindex.size(); ++c) uimg[c] = h.uindex[c] > -1 ? h.u[(size_t)h.uindex[c]] : 0.0;
    if (vimg) for (size_t c = 0; c < N; ++c) vimg[c] = h.vindex[c] > -1 ? h.v[(size_t)h.vindex[c]] : 0.0;
    if (wimg) for (size_t c = 0; c < N; ++c) wimg[c] = h.windex[c] > -1 ? h.w[(size_t)h.windex[c]] : 0.0;
    if (vavg) {
        // face averages, src/NSBase.cxx:425-466
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k) {
                    size_t c = ((size_t)i * ny + j) * nz + k;
                    double au = 0, av = 0, aw = 0;
                    int a = h.Um(i + 1, j, k), b = h.Um(i, j, k);
                    if (a > -1 && b > -1) au = (h.u[(size_t)a] + h.u[(size_t)b]) * 0.50;
                    else if (a > -1) au = (h.u[(size_t)a]) * 0.50;
                    else if (b > -1) au = (h.u[(size_t)b]) * 0.50;
                    b = h.Vm(i, j, k);
                    if (j < ny - 1) {
                        a = h.Vm(i, j + 1, k);
                        if (a > -1 && b > -1) av = (h.v[(size_t)a] + h.v[(size_t)b]) * 0.50;
                        else if (a > -1) av = (h.v[(size_t)a]) * 0.50;
                        else if (b > -1) av = (h.v[(size_t)b]) * 0.50;
                    } else if (b > -1) av = (h.v[(size_t)b]) * 0.50;
                    b = h.Wm(i, j, k);
                    if (k < nz - 1) {
                        a = h.Wm(i, j, k + 1);
                        if (a > -1 && b > -1) aw = (h.w[(size_t)a] + h.w[(size_t)b]) * 0.50;
                        else if (a > -1) aw = (h.w[(size_t)a]) * 0.50;
                        else if (b > -1) aw = (h.w[(size_t)b]) * 0.50;
                    } else if (b > -1) aw = (h.w[(size_t)b]) * 0.50;
                    vavg[3 * c + 0] = au; vavg[3 * c + 1] = av; vavg[3 * c + 2] = aw;
                }
    }
    return NS3D_OK;
}

NS3D_API int ns3d_set_output(ns3d_handle *H, const char *dir, const char *stem, int32_t write_fields) {
    (void)write_fields;
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    h.info.close();
    h.resl.close();
    h.have_out = false;
    if (!dir) return NS3D_OK;
    h.outdir = dir;
    h.stem = stem ? stem : "image";
    std::string d = h.outdir.empty() ? std::string() : h.outdir + "/";
    std::string in = d + "INFO-" + std::to_string(h.prm.direction) + "-" + h.stem + ".log";
    std::string rn = d + "RES-" + std::to_string(h.prm.direction) + "-" + h.stem + ".csv";
    h.info.f = fopen(in.c_str(), "w");
    h.resl.f = fopen(rn.c_str(), "w");
    if (!h.info.f || !h.resl.f) return fail(NS3D_ERR_IO, "cannot open log files in %s", dir);
    h.info.prec = 15;
    h.resl.prec = 6;
    h.have_out = true;
    // constructor lines that reach the file, src/NSBase.cxx:143,182-187
    h.info.s("Size "); h.info.i(h.nx); h.info.s(","); h.info.i(h.ny); h.info.s(","); h.info.i(h.nz); h.info.nl();
    h.info.s("Porosity: "); h.info.d((double)(float(h.np) / float((long)h.nx * h.ny * h.nz))); h.info.nl();
    h.info.s("Nodes for the pressure field: "); h.info.i(h.np); h.info.nl();
    h.info.s("Nodes for the u velocity field: "); h.info.i(h.nu); h.info.nl();
    h.info.s("Nodes for the v velocity field: "); h.info.i(h.nv); h.info.nl();
    h.info.s("Nodes for the w velocity field: "); h.info.i(h.nw); h.info.nl();
    h.info.s("Delta RMR min : "); h.info.d(h.deltaRMR); h.info.nl();
    return NS3D_OK;
}

/* Oracle only (not in the header): wall seconds of the last ns3d_solve per
 * phase -- out[0] assembly, out[1] BiCGSTAB solves, out[2] corrections,
 * out[3] diagnostics. */
NS3D_API int ns3d_oracle_phase_seconds(double *out) {
    if (!out) return fail(NS3D_ERR_ARG, "NULL output");
    for (int i = 0; i < 4; ++i) out[i] = g_phase_s[i];
    return NS3D_OK;
}

NS3D_API int ns3d_solve(ns3d_handle *H) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    std::memset(&h.res, 0, sizeof h.res);
    h.su = h.sv = h.sw = h.sp = SolveOut();
    h.alpha = h.alpha0;
    h.beta = h.beta0;
    h.avgRMR.clear();
    h.RMR = h.old_RMR = 0;
    for (double &t : g_phase_s) t = 0.0;
    switch (h.prm.method) {
        case NS3D_SIMPLEC: run_simplec(h); break;
        case NS3D_SIMPLER:
        case NS3D_SIMPLERR:
        case NS3D_IDEAL: run_simpler_family(h, h.prm.method); break;
        default: return fail(NS3D_ERR_ARG, "unknown method %d", h.prm.method);
    }
    return NS3D_OK;
}

NS3D_API int ns3d_get_result(const ns3d_handle *H, ns3d_result *r) {
    if (!H || !r) return fail(NS3D_ERR_ARG, "NULL argument");
    *r = H->h.res;
    return NS3D_OK;
}

NS3D_API int ns3d_assemble_momentum(ns3d_handle *H) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    assemble_all_momentum(h, h.u, h.v, h.w);
    rhs_u(h);
    rhs_v(h);
    if (h.nw > 0) rhs_w(h);
    return NS3D_OK;
}

NS3D_API int ns3d_assemble_pressure_correction(ns3d_handle *H, int32_t simplec) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    assemble_pressure_system(h, simplec ? 1 : 2, false, h.u, h.v, h.w);
    return NS3D_OK;
}

NS3D_API int ns3d_assemble_pressure(ns3d_handle *H, int32_t relax) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    std::vector<double> uh, vh, wh;
    compute_hat(h, h.U, h.u, h.u, uh);
    compute_hat(h, h.V, h.v, h.v, vh);
    compute_hat(h, h.W, h.w, h.w, wh);
    assemble_pressure_system(h, 0, relax != 0, uh, vh, wh);
    return NS3D_OK;
}

NS3D_API int ns3d_get_system(ns3d_handle *H, int32_t sys, double *coef, int32_t *nbr, double *rhs, double *rowsum) {
    if (!H) return fail(NS3D_ERR_ARG, "NULL handle");
    Handle &h = H->h;
    System *S = sys == NS3D_SYS_U ? &h.U : sys == NS3D_SYS_V ? &h.V : sys == NS3D_SYS_W ? &h.W : sys == NS3D_SYS_P ? &h.P : nullptr;
    if (!S) return fail(NS3D_ERR_ARG, "bad system %d", sys);
    const size_t n = (size_t)S->n;
    if (coef)
        for (int s = 0; s < 7; ++s) std::memcpy(coef + s * n, S->c[s].data(), n * 8);
    if (nbr)
        for (int s = 0; s < 6; ++s) std::memcpy(nbr + s * n, S->nb[s].data(), n * 4);
    if (rhs) std::memcpy(rhs, S->rhs.data(), n * 8);
    if (rowsum) std::memcpy(rowsum, S->rowsum.data(), n * 8);
    return NS3D_OK;
}

NS3D_API int ns3d_solve_system(ns3d_handle *H, int32_t sys, const double *rhs, double *x, double tol, int32_t maxit,
                               ns3d_solve_info *info) {
    if (!H || !x) return fail(NS3D_ERR_ARG, "NULL argument");
    Handle &h = H->h;
    System *S = sys == NS3D_SYS_U ? &h.U : sys == NS3D_SYS_V ? &h.V : sys == NS3D_SYS_W ? &h.W : sys == NS3D_SYS_P ? &h.P : nullptr;
    if (!S) return fail(NS3D_ERR_ARG, "bad system %d", sys);
    std::vector<double> b = rhs ? std::vector<double>(rhs, rhs + S->n) : S->rhs;
    std::vector<double> xx(x, x + S->n);
    SolveOut o = bicgstab(*S, b, xx, tol, maxit, nullptr);
    std::memcpy(x, xx.data(), xx.size() * 8);
    if (info) { info->iterations = (int32_t)o.iters; info->info = o.info; info->error = o.error; }
    return NS3D_OK;
}

NS3D_API int ns3d_close(ns3d_handle *H) {
    delete H;
    return NS3D_OK;
}

}  // extern "C"
