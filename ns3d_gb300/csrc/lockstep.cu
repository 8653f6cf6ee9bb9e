// lockstep.cu -- the SIMPLEC solves of many images driven together from one
// host thread (ns3d_solve_lockstep, ns3d_batch_solve_lockstep).
//
// Every image keeps its own solver instance (fields, systems, relaxation
// state, logs) and takes exactly the steps of SIMPLECSOLVER::Solve
// (src/SIMPLEC.cxx:73-232) in the order of ns3d_handle::run_simplec.  The
// driver runs each step for all running images before the next step:
//  * every image's kernels go to one stream, in image order;
//  * each BiCGSTAB step is solved as merged sets (the momentum systems of all
//    images, then their pressure-correction systems), one persistent
//    loop-kernel launch per round over the ragged chunk list of all of them,
//    FP64 or FP32 inside FP64 defect correction by each image's precision;
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

    // items[i]: member i's systems (its momentum set or its pressure set);
    // on return outs[i] holds their outcomes and the member's own set holds
    // their final states (read by the member's later kernels)
    void solve(const std::vector<Member *> &ms, std::vector<std::vector<SolveItem>> &items, bool momentum,
               std::vector<std::vector<SolveOutcome>> &outs) {
        const int n = (int)ms.size();
        outs.assign(n, {});
        std::vector<int> fp64, mixed[2];
        for (int i = 0; i < n; ++i) {
            ns3d_handle &h = *ms[i]->h;
            if (!h.mixed()) {
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
    std::vector<std::vector<SolveItem>> items;
    for (Member *m : ms) items.push_back(m->h->velocity_begin());
    std::vector<std::vector<SolveOutcome>> outs;
    solver.solve(ms, items, true, outs);
    for (size_t i = 0; i < ms.size(); ++i) ms[i]->h->velocity_end(outs[i], limit, dvmax(*ms[i]));
}

// SIMPLECSOLVER::Solve (src/SIMPLEC.cxx:73-232) for every member, step by
// step, in the order of ns3d_handle::run_simplec
void run_lockstep(std::vector<Member> &all, cudaStream_t st) {
    StepSolver solver(st);
    std::vector<Member *> run;
    for (Member &m : all) {
        m.t0 = Clock::now();
        m.start = time(0);
        m.h->header("SIMPLEC", "Max number of SIMPLE iterations: ");
        m.h->alpha = m.h->alpha0;
        run.push_back(&m);
    }
    // initial velocity and permeability
    for (Member *m : run) m->h->assemble_all_momentum();
    velocity_step(solver, run, false, [](const Member &) { return 0.0; });
    for (Member *m : run) m->h->permeability_launch();
    for (Member *m : run) {
        m->h->permeability_read(m->s);
        m->h->info.s("Initial Permeability K (m²): ").d(m->s.K).nl();
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
        if (it > 0) {
            for (Member *m : run) m->h->assemble_all_momentum();
            velocity_step(solver, run, true, [](const Member &m) {
                return m.s.v_moy * std::min(1., m.h->alpha * 1.5);
            });
        }
        for (Member *m : run) m->h->permeability_launch();
        for (Member *m : run) m->h->permeability_read(m->s);
        for (Member *m : run) m->h->divergence_launch();
        for (Member *m : run) m->h->divergence_read(m->s);
        std::vector<Member *> cont;
        for (Member *m : run) {
            ns3d_handle &h = *m->h;
            h.diagnostics_end(m->s);
            h.old_rmr_update(it);
            h.res_row(it, m->s);
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
        std::vector<std::vector<SolveItem>> items;
        for (Member *m : run) {
            ns3d_handle &h = *m->h;
            const Grid g = h.grid();
            const Phys ph = h.phys();
            launch_assemble_pressure(1, 0, g, ph, h.P.view(), h.U.view(), h.V.view(), h.W.view(), h.u.p, h.v.p,
                                     h.w.p, h.p.p, h.stream);
            items.push_back(h.pressure_correction_begin());
        }
        std::vector<std::vector<SolveOutcome>> outs;
        solver.solve(run, items, false, outs);
        for (size_t i = 0; i < run.size(); ++i) {
            ns3d_handle &h = *run[i]->h;
            h.pressure_correction_end(outs[i]);
            const Grid g = h.grid();
            const Phys ph = h.phys();
            const double dvmax = run[i]->s.v_moy * h.alpha;
            launch_correct_velocity(0, 1, g, ph, h.U.view(), h.pc.p, h.u.p, dvmax, h.stream);
            launch_correct_velocity(1, 1, g, ph, h.V.view(), h.pc.p, h.v.p, dvmax, h.stream);
            if (h.nw > 0) launch_correct_velocity(2, 1, g, ph, h.W.view(), h.pc.p, h.w.p, dvmax, h.stream);
            h.correct_pressure_launch();
        }
        for (Member *m : run) m->h->correct_pressure_read();
        for (Member *m : run) m->h->divergence_launch();
        for (Member *m : run) {
            ns3d_handle &h = *m->h;
            Scalars after = m->s;
            h.divergence_read(after);
            m->s.MaxDeltaV = after.MaxDeltaV;
            m->s.normdiv = after.normdiv;
            m->s.velocityNorm = after.velocityNorm;
            m->s.maxdiv = after.maxdiv;
            h.save_snapshot(it, m->savecounter);
            h.relax_control(true);
        }
    }
    for (Member &m : all) m.h->finish("SIMPLEC", m.it, m.s, m.t0, m.start);
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
        h.begin_solve();
        // set-up that allocates (state buffers, FP32 copies, multilevel
        // hierarchy) happens on the instance's own stream: its buffers are
        // freed there later
        const std::vector<SolveItem> mom = h.momentum_items(), pcs = h.pressure_correction_items();
        if (h.mixed()) {
            h.mmom.prepare(mom, h.stream);
            h.mp.prepare(pcs, h.stream);
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
