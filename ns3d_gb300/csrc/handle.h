// handle.h -- the solver instance behind the C-ABI handle (ns3d_handle):
// device state of one image, the steps of the reference's drivers as
// methods, and its logs.  Defined in solver.cu; the lockstep driver
// (lockstep.cu) runs the steps of many instances together.
#pragma once

#include <chrono>
#include <ctime>
#include <list>
#include <string>
#include <vector>

#include "hostio.h"
#include "runtime.h"

namespace ns3d {

struct Scalars {
    double Q = 0, v_moy = 0, K = 0, normdiv = 0, reldiv = 0, velocityNorm = 0, maxdiv = 0, MaxDeltaV = 0;
};

}  // namespace ns3d

struct ns3d_handle {
    ns3d_params prm;
    int rnx = 0, rny = 0, rnz = 0;  // raw image
    int nx = 0, ny = 0, nz = 0;     // solver frame
    int np = 0, nu = 0, nv = 0, nw = 0;
    ns3d::OwnedStream owned_stream;  // destroyed after every buffer freed on it
    cudaStream_t stream = nullptr;

    ns3d::DBuf<uint8_t> img;
    ns3d::DBuf<int> pmap, umap, vmap, wmap;
    ns3d::DevSys U, V, W, P;
    // fields and work vectors (npad of their system)
    ns3d::DBuf<double> p, u, v, w, pc, ptemp, utemp, vtemp, wtemp, uh, vh, wh, ut, vt, wt;
    ns3d::DBuf<double> diag_part;
    ns3d::DBuf<ns3d::DiagOut> diag;
    ns3d::HBuf<ns3d::DiagOut> h_diag;
    ns3d::KrylovSet kmom, kp;
    ns3d::MixedSet mmom, mp;  // FP32 inner / FP64 outer solves (precision = MIXED)
    ns3d::SolveGroup *group = nullptr;  // sets merged with other solves' (ns3d_set_group)
    bool mixed() const { return prm.precision != NS3D_FP64; }
    // an FP64 set: alone, or merged with the sets of the group's other solves
    void run_fp64(ns3d::KrylovSet &own, const std::vector<ns3d::SolveItem> &items,
                  std::vector<ns3d::SolveOutcome> &out) {
        if (!group) {
            own.run(items, stream, out);
            return;
        }
        own.prepare(items, stream);  // the merged run leaves the final states here
        group->run(items, stream, own.state_buffer(), out);
    }
    // a mixed-precision set: alone, or merged (with the preconditioner and
    // FP32 loop variant its own set chooses)
    void run_mixed(ns3d::MixedSet &own, std::vector<ns3d::SolveItem> items, std::vector<ns3d::SolveOutcome> &out) {
        if (!group) {
            own.run(items, stream, out);
            return;
        }
        own.prepare(items, stream);  // FP32 copies, hierarchy, outcome states
        for (size_t i = 0; i < items.size(); ++i) items[i].mg = own.uses_mg((int)i);
        group->run_mixed(items, stream, own.out_state_buffer(), out, own.variant());
    }
    // A pressure(-correction) solve.  In the mixed modes a solve that ends
    // without success (no convergence within the iteration cap, or a
    // numerical breakdown of the FP32 inner solves -- on strongly fragmented
    // pore spaces, whose many isolated clusters give singular blocks, the
    // FP32 solves stall) is redone in plain FP64 from the guess it started
    // from, and the rest of this solve's pressure systems go straight to
    // FP64.  The reported outcome is the FP64 solve's; both solves' work is
    // counted.
    bool p_fp64 = false;  // reset by begin_solve
    ns3d::DBuf<double> p_guess;
    void solve_p(const std::vector<ns3d::SolveItem> &items, std::vector<ns3d::SolveOutcome> &out) {
        if (!mixed() || p_fp64) {
            run_fp64(kp, items, out);
            return;
        }
        const ns3d::DevSys &S = *items[0].sys;
        if (p_guess.n < (size_t)S.npad) p_guess.alloc(S.npad, stream);
        NS3D_CUDA_CHECK(cudaMemcpyAsync(p_guess.p, items[0].x, (size_t)S.npad * 8, cudaMemcpyDeviceToDevice, stream));
        run_mixed(mp, items, out);
        if (out[0].info == NS3D_SUCCESS) return;
        p_fallbacks += 1;
        p_fp64 = true;
        const int wasted = out[0].work;
        NS3D_CUDA_CHECK(cudaMemcpyAsync(items[0].x, p_guess.p, (size_t)S.npad * 8, cudaMemcpyDeviceToDevice, stream));
        run_fp64(kp, items, out);
        out[0].work += wasted;
    }
    int p_fallbacks = 0;  // mixed pressure solves redone in FP64 (reset by begin_solve)

    // physical constants and relaxation state (NavierStokesBase members)
    double dx, dy, dz, mu, rho, p0, p1, gradp, alpha0, beta0, alpha, beta;
    double p_inlet = 0, p_outlet = 0, schemefactor, min_alpha, min_beta, relax, speedup, maxconvdelta;
    double RMR = 0, old_RMR = 0, deltaRMR, pcmax = 0, pcmin = 0, pcnorm = 0;
    int border;
    std::list<double> avgRMR;
    ns3d::SolveOutcome su, sv, sw, sp;

    ns3d_result res;
    std::string outdir, stem;
    bool write_fields = false, have_out = false;
    ns3d::TextLog info, resl;

    ns3d::Grid grid() const {
        ns3d::Grid g;
        g.nx = nx; g.ny = ny; g.nz = nz;
        g.pmap = pmap.p; g.umap = umap.p; g.vmap = vmap.p; g.wmap = wmap.p;
        return g;
    }
    ns3d::Phys phys() const {
        ns3d::Phys ph;
        ph.dx = dx; ph.dy = dy; ph.dz = dz; ph.mu = mu; ph.rho = rho; ph.alpha = alpha; ph.beta = beta;
        ph.p0 = p0; ph.p1 = p1; ph.schemefactor = schemefactor;
        ph.idx = 1 / dx; ph.idy = 1 / dy; ph.idz = 1 / dz;
        ph.idx2 = 1 / (dx * dx); ph.idy2 = 1 / (dy * dy); ph.idz2 = 1 / (dz * dz);
        return ph;
    }

    // ---------------------------------------------------------------------
    void build(const uint8_t *raw, int rx, int ry, int rz);
    void default_fields();
    void set_pressure_drop(double p0_in, double gradp_in);
    void assemble_all_momentum();
    void momentum_rhs();
    void compute_velocity_field(bool limit, double dvmax);
    // the steps split where the lockstep driver solves or reads back for
    // many instances at once (the whole steps are these parts in order)
    void begin_solve();
    std::vector<ns3d::SolveItem> momentum_items();             // the u, v (, w) systems
    std::vector<ns3d::SolveItem> pressure_correction_items();  // the pc system
    std::vector<ns3d::SolveItem> velocity_begin();
    void velocity_end(const std::vector<ns3d::SolveOutcome> &out, bool limit, double dvmax);
    std::vector<ns3d::SolveItem> pressure_correction_begin();
    void pressure_correction_end(const std::vector<ns3d::SolveOutcome> &out);
    void correct_pressure_launch();
    void correct_pressure_read();
    void permeability_launch();
    void permeability_read(ns3d::Scalars &s);
    void divergence_launch();
    void divergence_read(ns3d::Scalars &s);
    void diagnostics_end(ns3d::Scalars &s);
    void log_solve(const char *comp, const ns3d::SolveOutcome &o);
    void log_pressure_status(const ns3d::SolveOutcome &o);
    void compute_pressure_correction();
    void compute_pressure_field();
    void correct_pressure_field();
    void permeability(ns3d::Scalars &s);
    void divergence(ns3d::Scalars &s);
    void diagnostics(ns3d::Scalars &s);
    void relax_control(bool beta_cst);
    bool check_convergence(double res_, double tol) const;
    void pressure_step(bool relax_p, const double *uc, const double *vc, const double *wc, const double *uold,
                       const double *vold, const double *wold, double *ux, double *vx, double *wx);
    void hats(const double *uc, const double *vc, const double *wc, const double *uold, const double *vold,
              const double *wold);
    void res_row(int it, const ns3d::Scalars &s);
    void fields_to_image(const std::string &file);
    void save_snapshot(int it, int &savecounter);
    void header(const char *name, const char *maxname);
    void finish(const char *name, int it, const ns3d::Scalars &s, std::chrono::steady_clock::time_point t0,
                time_t start);
    void initial_velocity(ns3d::Scalars &s);
    void run_simplec();
    void run_simpler_family(int method);
    void old_rmr_update(int it) {
        if (it > 1) {
            if (RMR < old_RMR) old_RMR = RMR;
        } else {
            old_RMR = RMR;
        }
    }
    void sync() { NS3D_CUDA_CHECK(cudaStreamSynchronize(stream)); }
    void d2d(double *dst, const double *src, size_t n) {
        if (n) NS3D_CUDA_CHECK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    }
};

// the SIMPLEC solves of n instances driven together (lockstep.cu); the
// arguments are checked by the caller; throws on failure
int lockstep_solve(ns3d_handle *const *hs, int n, int *status);
