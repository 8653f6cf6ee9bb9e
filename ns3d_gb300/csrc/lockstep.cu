// lockstep.cu -- the solves of many images driven together from one host
// thread (ns3d_solve_lockstep, ns3d_batch_solve_lockstep), any mix of the
// four methods.
//
// Every image keeps its own solver instance (fields, systems, relaxation
// state, logs) and takes exactly the steps of its method's driver in the
// order of ns3d_handle::run_simplec / run_simpler_family.  The driver runs
// each stage of an outer iteration for all running images before the next:
//  * every image's kernels go to one stream, in image order;
//  * each BiCGSTAB step is solved as merged sets (the momentum systems of all
//    images, then their pressure or pressure-correction systems), one
//    persistent loop-kernel launch per round over the ragged chunk list of
//    all of them, FP64 or FP32 inside FP64 defect correction by each image's
//    precision (with the FP64 redo of a failed mixed pressure solve that
//    ns3d_handle::solve_p makes);
//  * each reduction read-back waits for the stream once for all images (the
//    first image's read finds every image's reductions done).
// The host is thus synchronised a fixed number of times per outer iteration
// for the whole batch, instead of per image.  Each system keeps its own
// scalars, reduction order and preconditioner, so every image's result,
// logs included, is bit-identical to its own ns3d_solve.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <ctime>
#include <vector>

#include "handle.h"
#include "runtime.h"

namespace {

using namespace ns3d;
using Clock = std::chrono::steady_clock;

struct Member {
    ns3d_handle *h = nullptr;
    int method = NS3D_SIMPLEC;
    bool simplec() const { return method == NS3D_SIMPLEC; }
    Scalars s;
    int savecounter = 0;
    int it = 0;  // the loop index when its solve ended ("terminated in N iteration")
    bool running = true;
    Clock::time_point t0;
    time_t start = 0;
    cudaStream_t own = nullptr;  // the instance's stream, restored at the end
};

// The merged solves of one BiCGSTAB step of the running images.
class StepSolver {
  public:
    explicit StepSolver(cudaStream_t st) : st_(st) {}

    // items[i]: member i's systems (its momentum set or its pressure set),
    // solved in FP64 where fp64[i], else in mixed precision; on return
    // outs[i] holds their outcomes and the member's own set holds their final
    // states (read by the member's later kernels)
    void solve(const std::vector<Member *> &ms, std::vector<std::vector<SolveItem>> &items, bool momentum,
               const std::vector<char> &use_fp64, std::vector<std::vector<SolveOutcome>> &outs) {
        const int n = (int)ms.size();
        outs.assign(n, {});
        std::vector<int> fp64, mixed[2];
        for (int i = 0; i < n; ++i) {
            ns3d_handle &h = *ms[i]->h;
            if (use_fp64[i]) {
                (momentum ? h.kmom : h.kp).prepare(items[i], st_);
                fp64.push_back(i);
            } else {
                MixedSet &own = momentum ? h.mmom : h.mp;
                own.prepare(items[i], st_);
                for (size_t k = 0; k < items[i].size(); ++k) items[i][k].mg = own.uses_mg((int)k);
                mixed[own.variant()].push_back(i);
            }
        }
        packed(fp64, KMAX_MERGED, items, outs, [&](const std::vector<SolveItem> &all, std::vector<SolveOutcome> &o) {
            kset_.run(all, st_, o);
        }, [&](int i, int off, int cnt) {
            ns3d_handle &h = *ms[i]->h;
            copy_states((momentum ? h.kmom : h.kp).state_buffer(), kset_.device_state(off), cnt);
        });
        for (int v = 0; v < 2; ++v)
            packed(mixed[v], KMAX_MERGED_M, items, outs,
                   [&](const std::vector<SolveItem> &all, std::vector<SolveOutcome> &o) { mset_.run(all, st_, o, v); },
                   [&](int i, int off, int cnt) {
                       ns3d_handle &h = *ms[i]->h;
                       copy_states((momentum ? h.mmom : h.mp).out_state_buffer(), mset_.device_state(off), cnt);
                   });
    }

  private:
    void copy_states(KState *dst, const KState *src, int cnt) {
        if (cnt)
            NS3D_CUDA_CHECK(cudaMemcpyAsync(dst, src, cnt * sizeof(KState), cudaMemcpyDeviceToDevice, st_));
    }
    // the members `idx` in order, as few merged sets as fit `cap` systems
    template <class Run, class Copy>
    void packed(const std::vector<int> &idx, int cap, const std::vector<std::vector<SolveItem>> &items,
                std::vector<std::vector<SolveOutcome>> &outs, Run run, Copy copy) {
        size_t a = 0;
        while (a < idx.size()) {
            std::vector<SolveItem> all;
            size_t b = a;
            while (b < idx.size() && (b == a || (int)(all.size() + items[idx[b]].size()) <= cap)) {
                all.insert(all.end(), items[idx[b]].begin(), items[idx[b]].end());
                ++b;
            }
            std::vector<SolveOutcome> o;
            run(all, o);
            int off = 0;
            for (size_t k = a; k < b; ++k) {
                const int i = idx[k], cnt = (int)items[i].size();
                outs[i].assign(o.begin() + off, o.begin() + off + cnt);
                copy(i, off, cnt);
                off += cnt;
            }
            a = b;
        }
    }

    cudaStream_t st_;
    KrylovSetMerged kset_;
    MixedSetMerged mset_;
};

// ComputeVelocityField of every member (the momentum assembly was launched)
template <class Dvmax>
void velocity_step(StepSolver &solver, const std::vector<Member *> &ms, bool limit, Dvmax dvmax) {
    if (ms.empty()) return;
    std::vector<std::vector<SolveItem>> items;
    std::vector<char> fp64;
    for (Member *m : ms) {
        items.push_back(m->h->velocity_begin());
        fp64.push_back(!m->h->mixed());
    }
    std::vector<std::vector<SolveOutcome>> outs;
    solver.solve(ms, items, true, fp64, outs);
    for (size_t i = 0; i < ms.size(); ++i) ms[i]->h->velocity_end(outs[i], limit, dvmax(*ms[i]));
}

// ns3d_handle::solve_p of every member: the mixed-precision pressure solves
// that end without success are redone in FP64 from the guess they started
// from (and the member's later pressure solves go straight to FP64)
void pressure_solve(StepSolver &solver, const std::vector<Member *> &ms, std::vector<std::vector<SolveItem>> &items,
                    std::vector<std::vector<SolveOutcome>> &outs) {
    const size_t n = ms.size();
    std::vector<char> fp64(n);
    for (size_t i = 0; i < n; ++i) {
        ns3d_handle &h = *ms[i]->h;
        fp64[i] = !h.mixed() || h.p_fp64;
        if (!fp64[i]) h.d2d(h.p_guess.p, items[i][0].x, (size_t)items[i][0].sys->npad);
    }
    solver.solve(ms, items, false, fp64, outs);
    std::vector<Member *> redo;
    std::vector<std::vector<SolveItem>> redo_items;
    std::vector<size_t> at;
    std::vector<int> wasted;
    for (size_t i = 0; i < n; ++i) {
        ns3d_handle &h = *ms[i]->h;
        if (fp64[i] || outs[i][0].info == NS3D_SUCCESS) continue;
        h.p_fallbacks += 1;
        h.p_fp64 = true;
        h.d2d(items[i][0].x, h.p_guess.p, (size_t)items[i][0].sys->npad);
        redo.push_back(ms[i]);
        redo_items.push_back(items[i]);
        at.push_back(i);
        wasted.push_back(outs[i][0].work);
    }
    if (redo.empty()) return;
    std::vector<std::vector<SolveOutcome>> again;
    solver.solve(redo, redo_items, false, std::vector<char>(redo.size(), 1), again);
    for (size_t k = 0; k < redo.size(); ++k) {
        outs[at[k]] = again[k];
        outs[at[k]][0].work += wasted[k];
    }
}

// ComputePressureField (src/NSBase.cxx:2383-2423) of every member whose
// pressure system is assembled: a solve that returns at once with success
// is retried with a tenth of the tolerance, member by member
void pressure_field(StepSolver &solver, const std::vector<Member *> &ms) {
    if (ms.empty()) return;
    std::vector<double> tol(ms.size());
    for (size_t i = 0; i < ms.size(); ++i) {
        ns3d_handle &h = *ms[i]->h;
        tol[i] = h.prm.psolvertol;
        h.info.s("Solving for pressure in : ");
        h.d2d(h.ptemp.p, h.p.p, h.P.npad);
    }
    std::vector<size_t> active(ms.size());
    for (size_t i = 0; i < ms.size(); ++i) active[i] = i;
    while (!active.empty()) {
        std::vector<Member *> sub;
        std::vector<std::vector<SolveItem>> items;
        for (size_t i : active) {
            ns3d_handle &h = *ms[i]->h;
            sub.push_back(ms[i]);
            items.push_back({{&h.P, h.ptemp.p, h.P.rhs.p, tol[i], h.prm.maxitsolver}});
        }
        std::vector<std::vector<SolveOutcome>> outs;
        pressure_solve(solver, sub, items, outs);
        std::vector<size_t> next;
        for (size_t k = 0; k < active.size(); ++k) {
            const size_t i = active[k];
            ns3d_handle &h = *ms[i]->h;
            h.sp = outs[k][0];
            h.res.krylov_iterations += h.sp.work;
            h.res.krylov_rows += (int64_t)h.sp.work * h.np;
            if (h.sp.iters == 0 && h.sp.info == NS3D_SUCCESS && tol[i] > 1e-15) {
                tol[i] *= 0.1;
                next.push_back(i);
            }
        }
        active.swap(next);
    }
    for (Member *m : ms) {
        ns3d_handle &h = *m->h;
        if (h.sp.iters > 0) h.d2d(h.p.p, h.ptemp.p, h.P.npad);
        h.log_pressure_status(h.sp);
    }
}

// Where the pressure step (ns3d_handle::pressure_step) reads its velocities
// and writes its corrected ones
struct PStepArgs {
    bool relax_p;
    const double *uc, *vc, *wc, *uold, *vold, *wold;
    double *ux, *vx, *wx;
};

// pseudo-velocities, pressure assembly, pressure solve, SIMPLER velocity
// correction of every member, each with its own arguments
void pressure_steps(StepSolver &solver, const std::vector<Member *> &ms, const std::vector<PStepArgs> &a) {
    if (ms.empty()) return;
    for (size_t i = 0; i < ms.size(); ++i) {
        ns3d_handle &h = *ms[i]->h;
        h.hats(a[i].uc, a[i].vc, a[i].wc, a[i].uold, a[i].vold, a[i].wold);
        launch_assemble_pressure(0, a[i].relax_p ? 1 : 0, h.grid(), h.phys(), h.P.view(), h.U.view(), h.V.view(),
                                 h.W.view(), h.uh.p, h.vh.p, h.wh.p, h.p.p, h.stream);
    }
    pressure_field(solver, ms);
    for (size_t i = 0; i < ms.size(); ++i) {
        ns3d_handle &h = *ms[i]->h;
        const Grid g = h.grid();
        const Phys ph = h.phys();
        launch_correct_velocity_simpler(0, g, ph, h.U.view(), h.p.p, h.uh.p, a[i].ux, h.p0, h.p1, h.stream);
        launch_correct_velocity_simpler(1, g, ph, h.V.view(), h.p.p, h.vh.p, a[i].vx, h.p0, h.p1, h.stream);
        if (h.nw > 0)
            launch_correct_velocity_simpler(2, g, ph, h.W.view(), h.p.p, h.wh.p, a[i].wx, h.p0, h.p1, h.stream);
    }
}

const char *method_name(int method) {
    return method == NS3D_SIMPLEC    ? "SIMPLEC"
           : method == NS3D_SIMPLER  ? "SIMPLER"
           : method == NS3D_SIMPLERR ? "SIMPLER-R"
                                     : "IDEAL";
}

// The outer loops of every member, one schedule for all four methods: each
// member takes exactly the steps of its own driver (SIMPLECSOLVER::Solve,
// src/SIMPLEC.cxx:73-232, as ns3d_handle::run_simplec; SIMPLERSOLVER,
// SIMPLERRSOLVER and IDEALSOLVER::Solve, src/SIMPLER.cxx:75-270,
// src/SIMPLERR.cxx:75-280, src/IDEAL.cxx:75-281, as
// ns3d_handle::run_simpler_family) in its order, and sits out the stages its
// method does not have.  Per outer iteration:
//   S1 momentum assembly (SIMPLEC from the second iteration on)
//   S2 N1 pressure steps (SIMPLER family)
//   S3 velocity solves (SIMPLEC from the second iteration on)
//   S4 permeability, divergence, RES row, convergence
//   S5 pressure-correction solve and velocity correction (all but IDEAL)
//   S6 pressure correction (SIMPLEC); pressure solve (SIMPLER-R); N2
//      pressure steps (IDEAL)
//   S7 divergence after the corrections, snapshot, relaxation control
void run_lockstep(std::vector<Member> &all, cudaStream_t st) {
    StepSolver solver(st);
    for (Member &m : all) {
        ns3d_handle &h = *m.h;
        m.t0 = Clock::now();
        m.start = time(0);
        if (m.simplec()) {
            h.header("SIMPLEC", "Max number of SIMPLE iterations: ");
            h.alpha = h.alpha0;
        } else {
            for (DBuf<double> *f : {&h.uh, &h.vh, &h.wh, &h.ut, &h.vt, &h.wt})
                if (f->n) NS3D_CUDA_CHECK(cudaMemsetAsync(f->p, 0, f->n * 8, h.stream));
            h.header(method_name(m.method), m.method == NS3D_SIMPLER    ? "Max number of SIMPLE iterations: "
                                            : m.method == NS3D_SIMPLERR ? "Max number of SIMPLE-R iterations: "
                                                                        : "Max number of IDEAL iterations: ");
        }
    }
    // initial velocity and permeability
    std::vector<Member *> run;
    for (Member &m : all) run.push_back(&m);
    for (Member *m : run) m->h->assemble_all_momentum();
    velocity_step(solver, run, false, [](const Member &) { return 0.0; });
    for (Member *m : run) m->h->permeability_launch();
    for (Member *m : run) {
        m->h->permeability_read(m->s);
        m->h->info.s("Initial Permeability K (m²): ").d(m->s.K).nl();
        if (!m->simplec()) m->h->alpha = m->h->alpha0;
    }
    for (int it = 0;; ++it) {
        run.clear();
        for (Member &m : all) {
            if (!m.running) continue;
            if (it < m.h->prm.maxitSIMPLE) {
                run.push_back(&m);
            } else {  // the loop of this image ends
                m.running = false;
                m.it = it;
            }
        }
        if (run.empty()) break;
        for (Member *m : run) m->h->info.s("Iteration ").i(it).s("  ------------").nl();
        // S1
        std::vector<Member *> vel;
        for (Member *m : run) {
            if (m->simplec() && it == 0) continue;
            ns3d_handle &h = *m->h;
            h.assemble_all_momentum();
            if (!m->simplec()) {
                h.d2d(h.ut.p, h.u.p, h.U.npad);
                h.d2d(h.vt.p, h.v.p, h.V.npad);
                if (h.nw > 0) h.d2d(h.wt.p, h.w.p, h.W.npad);
            }
            vel.push_back(m);
        }
        // S2
        for (int sub = 0;; ++sub) {
            std::vector<Member *> ms;
            std::vector<PStepArgs> a;
            for (Member *m : run) {
                ns3d_handle &h = *m->h;
                if (m->simplec() || sub >= h.prm.N1) continue;
                ms.push_back(m);
                a.push_back({true, h.ut.p, h.vt.p, h.wt.p, h.u.p, h.v.p, h.w.p, h.ut.p, h.vt.p, h.wt.p});
            }
            if (ms.empty()) break;
            pressure_steps(solver, ms, a);
        }
        // S3
        velocity_step(solver, vel, true, [](const Member &m) {
            return m.s.v_moy * std::min(1., m.h->alpha * 1.5);
        });
        // S4
        for (Member *m : run) m->h->permeability_launch();
        for (Member *m : run) m->h->permeability_read(m->s);
        for (Member *m : run) m->h->divergence_launch();
        for (Member *m : run) m->h->divergence_read(m->s);
        std::vector<Member *> cont;
        for (Member *m : run) {
            ns3d_handle &h = *m->h;
            h.diagnostics_end(m->s);
            h.old_rmr_update(it);
            if (m->method == NS3D_SIMPLEC || m->method == NS3D_SIMPLER) h.res_row(it, m->s);
            if (it > 1 && h.check_convergence(h.RMR, h.prm.simpletol)) {
                h.info.s("Permeability K (m²): ").d(m->s.K).nl();
                h.res.converged = 1;
                m->running = false;
                m->it = it;
            } else {
                cont.push_back(m);
            }
        }
        run.swap(cont);
        if (run.empty()) continue;
        // S5
        std::vector<Member *> pcm;
        std::vector<std::vector<SolveItem>> items;
        for (Member *m : run) {
            if (m->method == NS3D_IDEAL) continue;
            ns3d_handle &h = *m->h;
            launch_assemble_pressure(m->simplec() ? 1 : 2, 0, h.grid(), h.phys(), h.P.view(), h.U.view(), h.V.view(),
                                     h.W.view(), h.u.p, h.v.p, h.w.p, h.p.p, h.stream);
            items.push_back(h.pressure_correction_begin());
            pcm.push_back(m);
        }
        if (!pcm.empty()) {
            std::vector<std::vector<SolveOutcome>> outs;
            pressure_solve(solver, pcm, items, outs);
            for (size_t i = 0; i < pcm.size(); ++i) {
                ns3d_handle &h = *pcm[i]->h;
                h.pressure_correction_end(outs[i]);
                const Grid g = h.grid();
                const Phys ph = h.phys();
                const bool c = pcm[i]->simplec();
                const double dvmax = c ? pcm[i]->s.v_moy * h.alpha : pcm[i]->s.v_moy * 100;
                launch_correct_velocity(0, c, g, ph, h.U.view(), h.pc.p, h.u.p, dvmax, h.stream);
                launch_correct_velocity(1, c, g, ph, h.V.view(), h.pc.p, h.v.p, dvmax, h.stream);
                if (h.nw > 0) launch_correct_velocity(2, c, g, ph, h.W.view(), h.pc.p, h.w.p, dvmax, h.stream);
                if (c) h.correct_pressure_launch();
            }
        }
        // S6
        for (Member *m : pcm)
            if (m->simplec()) m->h->correct_pressure_read();
        std::vector<Member *> pf;
        for (Member *m : run) {
            ns3d_handle &h = *m->h;
            if (m->method == NS3D_SIMPLERR) {
                h.hats(h.u.p, h.v.p, h.w.p, h.u.p, h.v.p, h.w.p);
                launch_assemble_pressure(0, 1, h.grid(), h.phys(), h.P.view(), h.U.view(), h.V.view(), h.W.view(),
                                         h.uh.p, h.vh.p, h.wh.p, h.p.p, h.stream);
                pf.push_back(m);
            } else if (m->method == NS3D_IDEAL) {
                h.d2d(h.ut.p, h.u.p, h.U.npad);
                h.d2d(h.vt.p, h.v.p, h.V.npad);
                if (h.nw > 0) h.d2d(h.wt.p, h.w.p, h.W.npad);
            }
        }
        pressure_field(solver, pf);
        for (int sub = 0;; ++sub) {
            std::vector<Member *> ms;
            std::vector<PStepArgs> a;
            for (Member *m : run) {
                ns3d_handle &h = *m->h;
                if (m->method != NS3D_IDEAL || sub >= h.prm.N2) continue;
                ms.push_back(m);
                a.push_back({false, h.u.p, h.v.p, h.w.p, h.ut.p, h.vt.p, h.wt.p, h.u.p, h.v.p, h.w.p});
            }
            if (ms.empty()) break;
            pressure_steps(solver, ms, a);
        }
        // S7
        for (Member *m : run) m->h->divergence_launch();
        for (Member *m : run) {
            ns3d_handle &h = *m->h;
            Scalars after = m->s;
            h.divergence_read(after);
            m->s.MaxDeltaV = after.MaxDeltaV;
            m->s.normdiv = after.normdiv;
            m->s.velocityNorm = after.velocityNorm;
            m->s.maxdiv = after.maxdiv;
            if (m->method == NS3D_SIMPLERR) {
                h.res_row(it, m->s);
                h.relax_control(false);
                h.save_snapshot(it, m->savecounter);
            } else {
                h.save_snapshot(it, m->savecounter);
                h.relax_control(true);
            }
        }
    }
    for (Member &m : all) m.h->finish(method_name(m.method), m.it, m.s, m.t0, m.start);
}

}  // namespace

int lockstep_solve(ns3d_handle *const *hs, int n, int *status) {
    std::vector<Member> all((size_t)n);
    cudaStream_t st = nullptr;
    NS3D_CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct Restore {  // every instance gets its own stream back, the shared one is drained
        std::vector<Member> &all;
        cudaStream_t st;
        ~Restore() {
            cudaStreamSynchronize(st);
            for (Member &m : all)
                if (m.own) m.h->stream = m.own;
            cudaStreamDestroy(st);
        }
    } restore{all, st};
    for (int i = 0; i < n; ++i) {
        Member &m = all[(size_t)i];
        m.h = hs[i];
        ns3d_handle &h = *m.h;
        m.method = h.prm.method;
        h.begin_solve();
        // set-up that allocates (state buffers, FP32 copies, multilevel
        // hierarchy, the FP64 fallback's set and saved guess) happens on the
        // instance's own stream: its buffers are freed there later
        const std::vector<SolveItem> mom = h.momentum_items(), pcs = h.pressure_correction_items();
        if (h.mixed()) {
            h.mmom.prepare(mom, h.stream);
            h.mp.prepare(pcs, h.stream);
            h.kp.prepare(pcs, h.stream);
            if (h.p_guess.n < (size_t)h.P.npad) h.p_guess.alloc(h.P.npad, h.stream);
        } else {
            h.kmom.prepare(mom, h.stream);
            h.kp.prepare(pcs, h.stream);
        }
        NS3D_CUDA_CHECK(cudaStreamSynchronize(h.stream));
        m.own = h.stream;
        h.stream = st;
    }
    ActiveSolve active;
    run_lockstep(all, st);
    for (int i = 0; i < n; ++i)
        if (status) status[i] = NS3D_OK;
    return NS3D_OK;
}
