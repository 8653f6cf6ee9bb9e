// solver.cu -- host orchestration of the NS3D solve on one GB300 and the
// C-ABI of include/ns3d_capi.h.
//
// Everything inside the outer loop runs on the device (kernels in
// geometry.cu, physics.cu, krylov.cu); the host keeps the control flow of the
// reference drivers (SIMPLECSOLVER::Solve src/SIMPLEC.cxx:73-232,
// SIMPLERSOLVER::Solve src/SIMPLER.cxx:75-270, SIMPLERRSOLVER::Solve
// src/SIMPLERR.cxx:75-280, IDEALSOLVER::Solve src/IDEAL.cxx:75-281), the
// scalar relaxation state machine (RelaxControl, src/NSBase.cxx:196-301) and
// the INFO/RES logs.  Per outer iteration only a few scalars come back to the
// host: solver statuses, K, the divergence norms and the pressure-correction
// statistics.
#include <chrono>
#include <cmath>
#include <cstring>
#include <ctime>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "handle.h"
#include "hostio.h"
#include "runtime.h"
#include "tuner.h"

namespace ns3d {

// ============================ runtime =======================================
void DevSys::allocate(int rows, int first_extent, cudaStream_t st) {
    n = rows;
    npad = pad_rows(std::max(rows, 1));
    nchunks = (rows + CH - 1) / CH;
    d0 = first_extent;
    cell.alloc_zero(npad, st);
    coef.alloc_zero((size_t)7 * npad, st);
    nbr.alloc(6 * (size_t)npad, st);
    NS3D_CUDA_CHECK(cudaMemsetAsync(nbr.p, 0xff, nbr.n * sizeof(int), st));
    rhs.alloc_zero(npad, st);
    rowsum.alloc_zero(npad, st);
    invdiag.alloc_zero(npad, st);
    DBuf<double> *ws[] = {&r, &r0, &p, &v, &y, &s, &z, &t};
    for (auto *b : ws) b->alloc_zero(npad, st);
    part.alloc_zero((size_t)PART_PER_CHUNK * std::max(nchunks, 1), st);
}

size_t DevSys::device_bytes() const {
    return cell.n * 4 + coef.n * 8 + nbr.n * 4 + (rhs.n + rowsum.n + invdiag.n) * 8 + 8 * (size_t)npad * 8 +
           part.n * 8;
}

cudaMemPool_t device_pool() {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    NS3D_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw ApiError(NS3D_ERR_CUDA, "device index out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        NS3D_CUDA_CHECK(cudaMemPoolCreate(&pools[dev], &props));
        // keep released memory reserved for the next solves
        uint64_t keep = UINT64_MAX;
        NS3D_CUDA_CHECK(cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep));
    }
    return pools[dev];
}

size_t pool_cached_bytes() {
    cudaMemPool_t pool = device_pool();
    uint64_t reserved = 0, used = 0;
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
    cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
    return reserved > used ? (size_t)(reserved - used) : 0;
}

template <int CAP>
void KrylovSetT<CAP>::configure(const std::vector<SolveItem> &items, cudaStream_t st) {
    std::vector<KSys> ks;
    int chunk = 0;
    for (const SolveItem &it : items) {
        KSys k;
        DevSys &S = *it.sys;
        k.n = S.n;
        k.npad = S.npad;
        k.nchunks = S.nchunks;
        k.chunk_begin = chunk;
        chunk += S.nchunks;
        k.coef = S.coef.p;
        k.nbr = S.nbr.p;
        k.invdiag = S.invdiag.p;
        k.b = it.b;
        k.x = it.x;
        k.r = S.r.p; k.r0 = S.r0.p; k.p = S.p.p; k.v = S.v.p; k.y = S.y.p;
        k.s = S.s.p; k.z = S.z.p; k.t = S.t.p;
        k.part = S.part.p;
        k.st = nullptr;
        ks.push_back(k);
    }
    const int ns = (int)ks.size();
    if (ns > CAP) throw ApiError(NS3D_ERR_ARG, "too many systems in one solve set");
    if ((int)st_.n < ns) {
        st_.alloc_zero(ns, st);
        h_st_.alloc(ns);
        h_up_.alloc(ns);
    }
    if (!bar_.n) {
        bar_.alloc_zero(1, st);
        prof_.alloc_zero(1, st);
        h_err_.alloc(1);
        for (cudaEvent_t &e : ev_) NS3D_CUDA_CHECK(cudaEventCreate(&e));
    }
    std::memset(&set_, 0, sizeof set_);
    set_.nsys = ns;
    set_.total_chunks = chunk;
    for (int i = 0; i < ns; ++i) {
        ks[i].st = st_.p + i;
        set_.sys[i] = ks[i];
    }
    nsys_ = ns;
    total_chunks_ = chunk;
}

template <int CAP>
void KrylovSetT<CAP>::run(const std::vector<SolveItem> &items, cudaStream_t st,
                          std::vector<SolveOutcome> &out) {
    configure(items, st);
    const int ns = nsys_;
    out.assign(ns, SolveOutcome());
    int maxit = 0;
    for (int i = 0; i < ns; ++i) {
        KState z;
        std::memset(&z, 0, sizeof z);
        z.tol = items[i].tol;
        z.maxit = items[i].maxit;
        if (items[i].sys->n == 0) {  // no rows: nothing to launch, report like a zero right-hand side
            z.done = 1;
            z.zero_rhs = 1;
            z.iter = z.maxit;
            z.error = z.tol;
        }
        h_up_.p[i] = z;
        maxit = std::max(maxit, items[i].maxit);
    }
    NS3D_CUDA_CHECK(cudaMemcpyAsync(st_.p, h_up_.p, ns * sizeof(KState), cudaMemcpyHostToDevice, st));
    launch_krylov_init(set_, st);
    launches_ += 2;
    if (profiling) NS3D_CUDA_CHECK(cudaMemsetAsync(prof_.p, 0, sizeof(LoopProf), st));
    // The loop kernel runs until every system is done or one needs a
    // restart; restarts reset the iteration counter once, so 2*maxit+64
    // iterations bound the whole solve.
    const long cap = 2L * maxit + 64;
    long issued = 0;
    int loops = 0;
    std::vector<int> work_before(ns, 0);
    // merged sets: the grid of each loop launch comes from the autotuner,
    // which is told the launch's time per row-iteration
    const bool tune = CAP > KMAX;
    const uint64_t tkey = tuner_key(0, total_chunks_, share);
    int cand = 0;
    while (true) {
        NS3D_CUDA_CHECK(cudaMemcpyAsync(h_st_.p, st_.p, ns * sizeof(KState), cudaMemcpyDeviceToHost, st));
        NS3D_CUDA_CHECK(cudaMemcpyAsync(h_err_.p, &bar_.p->err, sizeof(int), cudaMemcpyDeviceToHost, st));
        NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
        // the flag belongs to this run's last loop launch (before the first
        // one it still holds the previous run's: a timed-out solve must not
        // poison the next)
        if (loops > 0 && h_err_.p[0])
            throw ApiError(NS3D_ERR_TIMEOUT, "BiCGSTAB loop kernel: a grid barrier timed out");
        bool all_done = true, any_paused = false;
        int progress = 0;
        int64_t rows = 0;
        for (int i = 0; i < ns; ++i) {
            const KState &k = h_st_.p[i];
            if (!k.done) all_done = false;
            if (k.paused && !k.done) any_paused = true;
            if (loops > 0) {
                progress = std::max(progress, k.work - work_before[i]);
                rows += (int64_t)set_.sys[i].n * (k.work - work_before[i]);
            }
            work_before[i] = k.work;
        }
        if (tune && loops > 0) {
            float ms = 0;
            NS3D_CUDA_CHECK(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
            grid_tuner().report(tkey, cand, ms, (double)rows);
        }
        if (profiling && loops > 0) {
            float ms = 0;
            NS3D_CUDA_CHECK(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
            prof.launches[5] += 1;
            prof.ms[5] += ms;
            prof.rows[5] += rows;
            for (int k = 0; k < 5; ++k) prof.rows[k] += rows;
        }
        issued += progress;
        if (all_done) break;
        if (loops > 0 && progress == 0 && !any_paused)
            throw ApiError(NS3D_ERR_TIMEOUT, "BiCGSTAB loop kernel made no progress");
        if (issued >= cap) throw ApiError(NS3D_ERR_TIMEOUT, "BiCGSTAB driver exceeded its iteration bound");
        if (any_paused) {
            launch_krylov_restart(set_, st);
            launches_ += 1;
        }
        if (tune) cand = grid_tuner().choose(tkey);
        if (profiling || tune) NS3D_CUDA_CHECK(cudaEventRecord(ev_[0], st));
        NS3D_CUDA_CHECK(launch_krylov_loop(set_, bar_.p, profiling ? prof_.p : nullptr, (int)(cap - issued), st,
                                           share << cand));
        if (profiling || tune) NS3D_CUDA_CHECK(cudaEventRecord(ev_[1], st));
        launches_ += 1;
        loops += 1;
    }
    if (profiling) {
        LoopProf lp;
        NS3D_CUDA_CHECK(cudaMemcpyAsync(&lp, prof_.p, sizeof lp, cudaMemcpyDeviceToHost, st));
        NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
        for (int k = 0; k < 5; ++k) {
            prof.ms[k] += 1e-6 * (double)lp.ns[k];
            prof.launches[k] += lp.iters;
        }
    }
    for (int i = 0; i < ns; ++i) {
        const KState &k = h_st_.p[i];
        out[i].iters = k.iter;
        out[i].info = k.info;
        out[i].error = k.error;
        out[i].work = k.work;
        out[i].valid = true;
    }
}

template <int CAP>
KrylovSetT<CAP>::~KrylovSetT() {
    for (cudaEvent_t e : ev_)
        if (e) cudaEventDestroy(e);
}

template class KrylovSetT<KMAX>;
template class KrylovSetT<KMAX_MERGED>;

// ============================ solver instance ================================
static thread_local std::string g_err;

static int set_error(int code, const std::string &m) {
    g_err = m;
    return code;
}

int report_error(int code, const std::string &m) { return set_error(code, m); }

}  // namespace ns3d

using namespace ns3d;

// ---- geometry -----------------------------------------------------------------
void ns3d_handle::build(const uint8_t *raw, int rx, int ry, int rz) {
    rnx = rx; rny = ry; rnz = rz;
    int ax = rx, ay = ry, az = rz;
    if (prm.direction == 2) std::swap(ax, ay);
    else if (prm.direction == 3) std::swap(ax, az);
    nx = ax + 2 * std::max(prm.border, 0);
    ny = ay;
    nz = az;
    const long N = (long)nx * ny * nz, NU = (long)(nx + 1) * ny * nz;
    if (NU > 0x7fffffffL) throw ApiError(NS3D_ERR_ARG, "image too large for int32 indices");
    DBuf<uint8_t> draw;
    draw.alloc((size_t)rx * ry * rz, stream);
    // host or device memory: the unified address space tells which
    NS3D_CUDA_CHECK(cudaMemcpyAsync(draw.p, raw, draw.n, cudaMemcpyDefault, stream));
    img.alloc(N, stream);
    launch_build_image(draw.p, rx, ry, rz, prm.direction, std::max(prm.border, 0), prm.porevalue, img.p, nx, ny, nz,
                       stream);
    pmap.alloc(N, stream); vmap.alloc(N, stream); wmap.alloc(N, stream); umap.alloc(NU, stream);
    for (DBuf<int> *m : {&pmap, &vmap, &wmap, &umap}) NS3D_CUDA_CHECK(cudaMemsetAsync(m->p, 0xff, m->n * 4, stream));
    // cell tables sized by the worst case, shrunk after the counts are known
    DBuf<int> pcell, ucell, vcell, wcell;
    pcell.alloc(N, stream); ucell.alloc(NU, stream); vcell.alloc(N, stream); wcell.alloc(N, stream);
    DBuf<int4> blk, tot;
    blk.alloc(index_build_blocks(N), stream);
    tot.alloc(1, stream);
    launch_index_build(img.p, nx, ny, nz, blk.p, tot.p, pmap.p, umap.p, vmap.p, wmap.p, pcell.p, ucell.p, vcell.p,
                       wcell.p, stream);
    int4 t;
    NS3D_CUDA_CHECK(cudaMemcpyAsync(&t, tot.p, sizeof(int4), cudaMemcpyDeviceToHost, stream));
    NS3D_CUDA_CHECK(cudaStreamSynchronize(stream));
    np = t.x; nu = t.y; nv = t.z; nw = t.w;
    U.allocate(nu, nx + 1, stream);
    V.allocate(nv, nx, stream);
    W.allocate(nw, nx, stream);
    P.allocate(np, nx, stream);
    P.cell_ny = ny;
    P.cell_nz = nz;
    NS3D_CUDA_CHECK(cudaMemcpyAsync(U.cell.p, ucell.p, (size_t)nu * 4, cudaMemcpyDeviceToDevice, stream));
    NS3D_CUDA_CHECK(cudaMemcpyAsync(V.cell.p, vcell.p, (size_t)nv * 4, cudaMemcpyDeviceToDevice, stream));
    NS3D_CUDA_CHECK(cudaMemcpyAsync(W.cell.p, wcell.p, (size_t)nw * 4, cudaMemcpyDeviceToDevice, stream));
    NS3D_CUDA_CHECK(cudaMemcpyAsync(P.cell.p, pcell.p, (size_t)np * 4, cudaMemcpyDeviceToDevice, stream));
    launch_nbr_mom(umap.p, nx + 1, ny, nz, U.cell.p, nu, U.npad, U.nbr.p, nz > 1, stream);
    launch_nbr_mom(vmap.p, nx, ny, nz, V.cell.p, nv, V.npad, V.nbr.p, nz > 1, stream);
    launch_nbr_mom(wmap.p, nx, ny, nz, W.cell.p, nw, W.npad, W.nbr.p, 1, stream);
    launch_nbr_p(grid(), P.cell.p, np, P.npad, P.nbr.p, stream);
    for (DBuf<double> *f : {&p, &pc, &ptemp}) f->alloc_zero(P.npad, stream);
    for (DBuf<double> *f : {&u, &utemp, &uh, &ut}) f->alloc_zero(U.npad, stream);
    for (DBuf<double> *f : {&v, &vtemp, &vh, &vt}) f->alloc_zero(V.npad, stream);
    for (DBuf<double> *f : {&w, &wtemp, &wh, &wt}) f->alloc_zero(W.npad, stream);
    int maxch = std::max({P.nchunks, (int)(((long)ny * nz + CH - 1) / CH), 1});
    diag_part.alloc_zero((size_t)5 * maxch, stream);
    diag.alloc_zero(1, stream);
    h_diag.alloc(1);
    NS3D_CUDA_CHECK(cudaStreamSynchronize(stream));  // temporaries are freed on return
}

// p0, gradp and the outlet pressure p1 = p0 - gradp dx nx, shifted so that
// p1 >= 0 (constructor, src/NSBase.cxx:155-161)
void ns3d_handle::set_pressure_drop(double p0_in, double gradp_in) {
    p0 = p0_in;
    gradp = gradp_in;
    p1 = -gradp * (dx * nx) + p0;
    if (p1 < 0) {
        p0 -= p1;
        p1 = 0;
    }
}

void ns3d_handle::default_fields() {
    for (DBuf<double> *f : {&p, &pc, &u, &v, &w})
        if (f->n) NS3D_CUDA_CHECK(cudaMemsetAsync(f->p, 0, f->n * 8, stream));
    launch_default_pressure(grid(), P.view(), p0, p1, p.p, stream);
}

// ---- momentum -------------------------------------------------------------------
// AssembleAllMomentum, src/NSBase.cxx:853-884 (the Jacobi factorization is
// the inverse diagonal, computed in the assembly epilogue with the row sums)
void ns3d_handle::assemble_all_momentum() {
    const Grid g = grid();
    const Phys ph = phys();
    launch_assemble_momentum(0, g, ph, U.view(), u.p, v.p, w.p, stream);
    launch_assemble_momentum(1, g, ph, V.view(), u.p, v.p, w.p, stream);
    if (nw > 0) launch_assemble_momentum(2, g, ph, W.view(), u.p, v.p, w.p, stream);
}

void ns3d_handle::momentum_rhs() {
    const Grid g = grid();
    const Phys ph = phys();
    launch_momentum_rhs(0, g, ph, U.view(), p.p, u.p, stream);
    launch_momentum_rhs(1, g, ph, V.view(), p.p, v.p, stream);
    if (nw > 0) launch_momentum_rhs(2, g, ph, W.view(), p.p, w.p, stream);
}

void ns3d_handle::log_solve(const char *comp, const SolveOutcome &o) {
    info.s("Solving for component ").s(comp).s(" in ").i(o.iters).s(" iterations (status ").i(o.info).s(")").nl();
}

// ComputeVelocityField, src/NSBase.cxx:1773-1884: the three components are
// solved together by one BiCGSTAB loop launch
void ns3d_handle::compute_velocity_field(bool limit, double dvmax) {
    const std::vector<SolveItem> items = velocity_begin();
    std::vector<SolveOutcome> out;
    if (mixed()) run_mixed(mmom, items, out);
    else run_fp64(kmom, items, out);
    velocity_end(out, limit, dvmax);
}

// the right-hand sides, the previous velocities, and the three systems
std::vector<SolveItem> ns3d_handle::velocity_begin() {
    momentum_rhs();
    d2d(utemp.p, u.p, U.npad);
    d2d(vtemp.p, v.p, V.npad);
    if (nw > 0) d2d(wtemp.p, w.p, W.npad);
    return momentum_items();
}

std::vector<SolveItem> ns3d_handle::momentum_items() {
    std::vector<SolveItem> items = {{&U, u.p, U.rhs.p, prm.vsolvertol, prm.maxitsolver},
                                    {&V, v.p, V.rhs.p, prm.vsolvertol, prm.maxitsolver}};
    if (nw > 0) items.push_back({&W, w.p, W.rhs.p, prm.vsolvertol, prm.maxitsolver});
    return items;
}

// revert or clamp each component by its solve's outcome; counts and logs
void ns3d_handle::velocity_end(const std::vector<SolveOutcome> &out, bool limit, double dvmax) {
    auto state = [&](int i) { return mixed() ? mmom.device_state(i) : kmom.device_state(i); };
    launch_velocity_post(utemp.p, u.p, nu, state(0), limit, dvmax, stream);
    launch_velocity_post(vtemp.p, v.p, nv, state(1), limit, dvmax, stream);
    if (nw > 0) launch_velocity_post(wtemp.p, w.p, nw, state(2), limit, dvmax, stream);
    su = out[0];
    sv = out[1];
    if (nw > 0) sw = out[2];
    for (const SolveOutcome &o : out) {
        res.krylov_iterations += o.work;
    }
    res.krylov_rows += (int64_t)su.work * nu + (int64_t)sv.work * nv + (nw > 0 ? (int64_t)sw.work * nw : 0);
    log_solve("u", su);
    log_solve("v", sv);
    if (nw > 0) log_solve("w", sw);
}

// ---- pressure ---------------------------------------------------------------------
void ns3d_handle::log_pressure_status(const SolveOutcome &o) {
    if (o.info == NS3D_SUCCESS) {
        info.i(o.iters).s(" iterations (status ").i(o.info).s(")").nl();
    } else {
        if (o.info == NS3D_NUMERICAL_ISSUE) info.s("Numerical Issue (iterations:").i(o.iters).s("). ");
        else if (o.info == NS3D_NO_CONVERGENCE) info.s("No convergence (iterations:").i(o.iters).s("). ");
        else if (o.info == NS3D_INVALID_INPUT) info.s("Invalid input (iterations:").i(o.iters).s("). ");
        info.s("Residual: ").d(o.error).nl();
    }
}

// ComputePressureCorrection, src/NSBase.cxx:2337-2365
void ns3d_handle::compute_pressure_correction() {
    const std::vector<SolveItem> items = pressure_correction_begin();
    std::vector<SolveOutcome> out;
    solve_p(items, out);
    pressure_correction_end(out);
}

std::vector<SolveItem> ns3d_handle::pressure_correction_begin() {
    info.s("Solving for pressure correction : ");
    return pressure_correction_items();
}

std::vector<SolveItem> ns3d_handle::pressure_correction_items() {
    return {{&P, pc.p, P.rhs.p, prm.pcsolvertol, prm.maxitsolver}};
}

void ns3d_handle::pressure_correction_end(const std::vector<SolveOutcome> &out) {
    sp = out[0];
    res.krylov_iterations += sp.work;
    res.krylov_rows += (int64_t)sp.work * np;
    log_pressure_status(sp);
}

// ComputePressureField, src/NSBase.cxx:2383-2423
void ns3d_handle::compute_pressure_field() {
    double tol = prm.psolvertol;
    info.s("Solving for pressure in : ");
    d2d(ptemp.p, p.p, P.npad);
    std::vector<SolveOutcome> out;
    solve_p({{&P, ptemp.p, P.rhs.p, tol, prm.maxitsolver}}, out);
    sp = out[0];
    res.krylov_iterations += sp.work;
    res.krylov_rows += (int64_t)sp.work * np;
    while (sp.iters == 0 && sp.info == NS3D_SUCCESS && tol > 1e-15) {
        tol *= 0.1;
        solve_p({{&P, ptemp.p, P.rhs.p, tol, prm.maxitsolver}}, out);
        sp = out[0];
        res.krylov_iterations += sp.work;
        res.krylov_rows += (int64_t)sp.work * np;
    }
    if (sp.iters > 0) d2d(p.p, ptemp.p, P.npad);
    log_pressure_status(sp);
}

// CorrectPressureField, src/NSBase.cxx:2367-2380
void ns3d_handle::correct_pressure_field() {
    correct_pressure_launch();
    correct_pressure_read();
}

void ns3d_handle::correct_pressure_launch() {
    launch_correct_pressure(P.view(), pc.p, p.p, beta, diag_part.p, diag.p, stream);
}

// Each *_read copies the reduction results to the host and waits for the
// stream: with many instances on one stream, the first read waits for every
// instance's launches and the others find them done.
void ns3d_handle::correct_pressure_read() {
    NS3D_CUDA_CHECK(cudaMemcpyAsync(h_diag.p, diag.p, sizeof(DiagOut), cudaMemcpyDeviceToHost, stream));
    sync();
    const DiagOut &d = *h_diag.p;
    pcmax = beta * d.pcmax;
    pcmin = beta * d.pcmin;
    pcnorm = beta * std::sqrt(d.pcsq);
    info.s("Correction de pression maximale et minimale: ").d(pcmax).s(", ").d(pcmin).nl();
    info.s("Norme de la correction de pression : ").d(pcnorm).nl();
}

// ---- diagnostics ------------------------------------------------------------------
// ComputePermeability, src/NSBase.cxx:1886-1956
void ns3d_handle::permeability(Scalars &s) {
    permeability_launch();
    permeability_read(s);
}

void ns3d_handle::permeability_launch() { launch_permeability(grid(), u.p, p.p, border, diag_part.p, diag.p, stream); }

void ns3d_handle::permeability_read(Scalars &s) {
    NS3D_CUDA_CHECK(cudaMemcpyAsync(h_diag.p, diag.p, sizeof(DiagOut), cudaMemcpyDeviceToHost, stream));
    sync();
    const DiagOut &d = *h_diag.p;
    const double sx = dy * dz;
    double v_moy = d.v_sum;
    if (border <= 0) {
        p_inlet = p0;
        p_outlet = p1;
    } else {
        p_inlet = d.p_in_sum;
        p_outlet = d.p_out_sum;
        int ci = (int)d.cnt_in, co = (int)d.cnt_out;
        if (ci > 0) p_inlet /= ci;
        if (co > 0) p_outlet /= co;
    }
    s.Q = v_moy * sx;
    v_moy /= (ny * nz);
    s.v_moy = v_moy;
    if (std::fabs(p_inlet - p_outlet) > 0.0)
        s.K = v_moy * mu * dx * (nx - 2 * border) / (p_inlet - p_outlet);
    else
        s.K = 0.0;
}

// ComputeDiv, src/NSBase.cxx:1958-2080
void ns3d_handle::divergence(Scalars &s) {
    divergence_launch();
    divergence_read(s);
}

void ns3d_handle::divergence_launch() {
    launch_divergence(grid(), phys(), P.view(), u.p, v.p, w.p, diag_part.p, diag.p, stream);
}

void ns3d_handle::divergence_read(Scalars &s) {
    NS3D_CUDA_CHECK(cudaMemcpyAsync(h_diag.p, diag.p, sizeof(DiagOut), cudaMemcpyDeviceToHost, stream));
    sync();
    const DiagOut &d = *h_diag.p;
    s.normdiv = std::sqrt(d.sumdiv2);
    s.velocityNorm = d.sumvel / np;
    s.maxdiv = d.maxdiv;
    s.MaxDeltaV = d.maxdv;
}

void ns3d_handle::diagnostics(Scalars &s) {
    permeability(s);
    divergence(s);
    diagnostics_end(s);
}

// RMR, relative divergence and the K line from the two reductions
void ns3d_handle::diagnostics_end(Scalars &s) {
    RMR = s.MaxDeltaV / std::fabs(s.v_moy);
    s.reldiv = (nx * dx + ny * dy + nz * dz) * s.maxdiv / (3 * s.v_moy);
    info.s("Permeability K (m²): ").d(s.K).nl();
}

// RelaxControl, src/NSBase.cxx:196-301
void ns3d_handle::relax_control(bool beta_cst) {
    const size_t size = 30;
    bool isDecreasing = false;
    if (RMR > old_RMR * maxconvdelta) {
        alpha = std::max(min_alpha, alpha - relax);
        if (!beta_cst) beta = std::max(min_beta, beta - relax);
        old_RMR *= 1.1;
        info.s("Relative Mass Residual increases too much -> new relaxation parameter alpha, beta: ").d(alpha).s(", ")
            .d(beta).nl();
        if (!avgRMR.empty()) avgRMR.pop_front();
    }
    if (!avgRMR.empty()) isDecreasing = avgRMR.back() > RMR;
    avgRMR.push_back(RMR);
    if (avgRMR.size() > size) {
        avgRMR.pop_front();
        int i = 0, n1 = 0, n2 = 0;
        double avg1 = 0, avg2 = 0;
        for (double x : avgRMR) {
            i += 1;
            if (i < avgRMR.size() * 0.5) { avg1 += x; n1 += 1; }
            else if (i >= avgRMR.size() * 0.5) { avg2 += x; n2 += 1; }
        }
        avg1 /= n1;
        avg2 /= n2;
        double delta = (avg2 - avg1) / std::max(avg1, avg2);
        if (delta <= 0 && std::fabs(delta) < deltaRMR && isDecreasing == false) {
            for (int c = 0; c < 15 && !avgRMR.empty(); ++c) avgRMR.pop_front();
            alpha = std::min(alpha0, alpha - relax * 0.25);
            if (!beta_cst) beta = std::max(min_beta, beta - relax * 0.25);
            info.s("Simulation is oscillating -> new relaxation parameter alpha, beta: ").d(alpha).s(", ").d(beta).nl();
        } else if (delta > 0 && isDecreasing == false) {
            for (int c = 0; c < 15 && !avgRMR.empty(); ++c) avgRMR.pop_front();
            alpha = std::max(min_alpha, alpha - relax);
            if (!beta_cst) beta = std::max(min_beta, beta - relax);
            info.s("Simulation is diverging -> new relaxation parameter alpha, beta: ").d(alpha).s(", ").d(beta).nl();
        }
    }
}

// CheckConvergence, src/NSBase.cxx:304-328
bool ns3d_handle::check_convergence(double r, double tol) const {
    if (r < tol) return true;
    return su.iters == 0 && sv.iters == 0 && (nw == 0 || sw.iters == 0) && sp.iters == 0;
}

// ---- SIMPLER-family building blocks -------------------------------------------------
void ns3d_handle::hats(const double *uc, const double *vc, const double *wc, const double *uold, const double *vold,
                       const double *wold) {
    const Phys ph = phys();
    launch_hat(U.view(), ph, uc, uold, uh.p, stream);
    launch_hat(V.view(), ph, vc, vold, vh.p, stream);
    if (nw > 0) launch_hat(W.view(), ph, wc, wold, wh.p, stream);
}

// Compute_*_hat; AssemblePressure; ComputePressureField;
// CorrectVelocityFieldSIMPLER into (ux, vx, wx)
void ns3d_handle::pressure_step(bool relax_p, const double *uc, const double *vc, const double *wc, const double *uold,
                                const double *vold, const double *wold, double *ux, double *vx, double *wx) {
    hats(uc, vc, wc, uold, vold, wold);
    const Grid g = grid();
    const Phys ph = phys();
    launch_assemble_pressure(0, relax_p ? 1 : 0, g, ph, P.view(), U.view(), V.view(), W.view(), uh.p, vh.p, wh.p,
                             p.p, stream);
    compute_pressure_field();
    launch_correct_velocity_simpler(0, g, ph, U.view(), p.p, uh.p, ux, p0, p1, stream);
    launch_correct_velocity_simpler(1, g, ph, V.view(), p.p, vh.p, vx, p0, p1, stream);
    if (nw > 0) launch_correct_velocity_simpler(2, g, ph, W.view(), p.p, wh.p, wx, p0, p1, stream);
}

// ---- logs and outputs ------------------------------------------------------------------
static const char *kResHeader =
    "iteration, Q (m³/s), <u_out> (m/s), Max Rel Mass Res., K (m²), gradP (Pa/m), ||Div_u||, "
    "Lref*(max DIV)/<u_out>, <||u||>, max DIV, it_u,it_v,it_w,it_pc";

void ns3d_handle::res_row(int it, const Scalars &s) {
    if (!resl.f) return;
    resl.i(it).s(",").d(s.Q).s(",").d(s.v_moy).s(",").d(RMR).s(",").d(s.K).s(",");
    resl.d((p_inlet - p_outlet) / (dx * (nx - 2 * border)));
    resl.s(",").d(s.normdiv).s(",").d(s.reldiv).s(",").d(s.velocityNorm).s(", ").d(s.maxdiv).s(", ");
    resl.i(su.valid ? su.iters : 0).s(",").i(sv.valid ? sv.iters : 0).s(",").i(sw.valid ? sw.iters : 0).s(",");
    resl.i(sp.valid ? sp.iters : 0).nl();
}

// FieldsToImage, src/NSBase.cxx:330-476
void ns3d_handle::fields_to_image(const std::string &file) {
    const char *pre[5] = {"Vx-", "Vy-", "Vz-", "V-", "P-"};
    std::string d = outdir.empty() ? std::string() : outdir + "/";
    if (have_out && write_fields) {
        const long N = (long)nx * ny * nz, NU = (long)(nx + 1) * ny * nz;
        DBuf<double> dimg;
        dimg.alloc((size_t)std::max(3 * N, NU), stream);
        std::vector<double> himg((size_t)std::max(3 * N, NU));
        std::string err, dir = std::to_string(prm.direction) + "-";
        auto dump = [&](const int *map, long cells, const double *f, int ex, const std::string &name) {
            launch_gather_image(map, cells, f, dimg.p, stream);
            NS3D_CUDA_CHECK(cudaMemcpyAsync(himg.data(), dimg.p, cells * 8, cudaMemcpyDeviceToHost, stream));
            sync();
            if (!vti_write_f64(d + name, himg.data(), ex, ny, nz, 1, err)) throw ApiError(NS3D_ERR_IO, err);
        };
        dump(umap.p, NU, u.p, nx + 1, std::string("Vx-") + dir + file);
        dump(vmap.p, N, v.p, nx, std::string("Vy-") + dir + file);
        dump(wmap.p, N, w.p, nx, std::string("Vz-") + dir + file);
        launch_face_average(grid(), u.p, v.p, w.p, dimg.p, stream);
        NS3D_CUDA_CHECK(cudaMemcpyAsync(himg.data(), dimg.p, 3 * N * 8, cudaMemcpyDeviceToHost, stream));
        sync();
        if (!vti_write_f64(d + "V-" + dir + file, himg.data(), nx, ny, nz, 3, err)) throw ApiError(NS3D_ERR_IO, err);
        dump(pmap.p, N, p.p, nx, std::string("P-") + dir + file);
    }
    for (auto pr : pre) info.s("Writing ").s(pr).i(prm.direction).s("-").s(file).nl();
}

void ns3d_handle::save_snapshot(int it, int &savecounter) {
    if (it % prm.save_step == 0 && it > 0) {
        savecounter += 1;
        if (savecounter > 3) savecounter = 1;
        fields_to_image(stem + "-SAVE-" + std::to_string(savecounter) + ".vti");
    }
}

void ns3d_handle::header(const char *name, const char *maxname) {
    info.s("Initializing ").s(name).s(" algorithm").nl();
    info.s("p0, p1 (Pa)= ").d(p0).s(",").d(p1).nl();
    info.s("Pressure gradient (Pa/m)= ").d((p0 - p1) / (dx * nx)).nl();
    info.s("inlet/outlet area (m²)= ").d(dy * dz * ny * nz).nl();
    info.s(maxname).i(prm.maxitSIMPLE).nl();
    if (resl.f) resl.s(kResHeader).nl();
}

void ns3d_handle::finish(const char *name, int it, const Scalars &s, std::chrono::steady_clock::time_point t0,
                         time_t start) {
    sync();
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    info.s("Norm of the velocity field divergence: ").d(s.normdiv).nl();
    info.s("Relative divergence of the velocity field: ").d(s.reldiv).nl();
    fields_to_image(stem + ".vti");
    time_t end = time(0);
    info.s(name).s(" terminated in ").i(it).s(" iteration and ").d(difftime(end, start)).s(" seconds").nl();
    ns3d_result &R = res;
    R.K = s.K; R.Q = s.Q; R.v_moy = s.v_moy; R.RMR = RMR;
    R.normdiv = s.normdiv; R.reldiv = s.reldiv; R.velocityNorm = s.velocityNorm; R.maxdiv = s.maxdiv;
    R.MaxDeltaV = s.MaxDeltaV; R.p_inlet = p_inlet; R.p_outlet = p_outlet; R.p0 = p0; R.p1 = p1;
    R.alpha = alpha; R.beta = beta; R.pcmax = pcmax; R.pcmin = pcmin; R.pcnorm = pcnorm;
    R.iterations = it;
    R.it_u = su.valid ? su.iters : 0;
    R.it_v = sv.valid ? sv.iters : 0;
    R.it_w = sw.valid ? sw.iters : 0;
    R.it_p = sp.valid ? sp.iters : 0;
    R.seconds = secs;
}

void ns3d_handle::initial_velocity(Scalars &s) {
    assemble_all_momentum();
    compute_velocity_field(false, 0);
    permeability(s);
    info.s("Initial Permeability K (m²): ").d(s.K).nl();
}

// SIMPLECSOLVER::Solve, src/SIMPLEC.cxx:73-232
void ns3d_handle::run_simplec() {
    auto t0 = std::chrono::steady_clock::now();
    time_t start = time(0);
    Scalars s;
    int savecounter = 0, it;
    header("SIMPLEC", "Max number of SIMPLE iterations: ");
    alpha = alpha0;
    initial_velocity(s);
    for (it = 0; it < prm.maxitSIMPLE; ++it) {
        info.s("Iteration ").i(it).s("  ------------").nl();
        if (it > 0) {
            assemble_all_momentum();
            compute_velocity_field(true, s.v_moy * std::min(1., alpha * 1.5));
        }
        diagnostics(s);
        old_rmr_update(it);
        res_row(it, s);
        if (it > 1 && check_convergence(RMR, prm.simpletol)) {
            info.s("Permeability K (m²): ").d(s.K).nl();
            res.converged = 1;
            break;
        }
        const Grid g = grid();
        const Phys ph = phys();
        launch_assemble_pressure(1, 0, g, ph, P.view(), U.view(), V.view(), W.view(), u.p, v.p, w.p, p.p, stream);
        compute_pressure_correction();
        const double dvmax = s.v_moy * alpha;
        launch_correct_velocity(0, 1, g, ph, U.view(), pc.p, u.p, dvmax, stream);
        launch_correct_velocity(1, 1, g, ph, V.view(), pc.p, v.p, dvmax, stream);
        if (nw > 0) launch_correct_velocity(2, 1, g, ph, W.view(), pc.p, w.p, dvmax, stream);
        correct_pressure_field();
        Scalars after = s;
        divergence(after);
        s.MaxDeltaV = after.MaxDeltaV; s.normdiv = after.normdiv; s.velocityNorm = after.velocityNorm;
        s.maxdiv = after.maxdiv;
        save_snapshot(it, savecounter);
        relax_control(true);
    }
    finish("SIMPLEC", it, s, t0, start);
}

// SIMPLERSOLVER::Solve src/SIMPLER.cxx:75-270, SIMPLERRSOLVER::Solve
// src/SIMPLERR.cxx:75-280, IDEALSOLVER::Solve src/IDEAL.cxx:75-281
void ns3d_handle::run_simpler_family(int method) {
    auto t0 = std::chrono::steady_clock::now();
    time_t start = time(0);
    Scalars s;
    int savecounter = 0, it;
    const char *name = method == NS3D_SIMPLER ? "SIMPLER" : method == NS3D_SIMPLERR ? "SIMPLER-R" : "IDEAL";
    const char *maxname = method == NS3D_SIMPLER    ? "Max number of SIMPLE iterations: "
                          : method == NS3D_SIMPLERR ? "Max number of SIMPLE-R iterations: "
                                                    : "Max number of IDEAL iterations: ";
    for (DBuf<double> *f : {&uh, &vh, &wh, &ut, &vt, &wt})
        if (f->n) NS3D_CUDA_CHECK(cudaMemsetAsync(f->p, 0, f->n * 8, stream));
    header(name, maxname);
    initial_velocity(s);
    alpha = alpha0;
    for (it = 0; it < prm.maxitSIMPLE; ++it) {
        info.s("Iteration ").i(it).s("  ------------").nl();
        assemble_all_momentum();
        d2d(ut.p, u.p, U.npad);
        d2d(vt.p, v.p, V.npad);
        if (nw > 0) d2d(wt.p, w.p, W.npad);
        for (int sub = 0; sub < prm.N1; ++sub)
            pressure_step(true, ut.p, vt.p, wt.p, u.p, v.p, w.p, ut.p, vt.p, wt.p);
        compute_velocity_field(true, s.v_moy * std::min(1., alpha * 1.5));
        diagnostics(s);
        old_rmr_update(it);
        if (method == NS3D_SIMPLER) res_row(it, s);
        if (it > 1 && check_convergence(RMR, prm.simpletol)) {
            info.s("Permeability K (m²): ").d(s.K).nl();
            res.converged = 1;
            break;
        }
        const Grid g = grid();
        Phys ph = phys();
        if (method == NS3D_SIMPLER || method == NS3D_SIMPLERR) {
            launch_assemble_pressure(2, 0, g, ph, P.view(), U.view(), V.view(), W.view(), u.p, v.p, w.p, p.p, stream);
            compute_pressure_correction();
            const double dvmax = s.v_moy * 100;
            launch_correct_velocity(0, 0, g, ph, U.view(), pc.p, u.p, dvmax, stream);
            launch_correct_velocity(1, 0, g, ph, V.view(), pc.p, v.p, dvmax, stream);
            if (nw > 0) launch_correct_velocity(2, 0, g, ph, W.view(), pc.p, w.p, dvmax, stream);
            if (method == NS3D_SIMPLERR) {
                hats(u.p, v.p, w.p, u.p, v.p, w.p);
                launch_assemble_pressure(0, 1, g, ph, P.view(), U.view(), V.view(), W.view(), uh.p, vh.p, wh.p, p.p,
                                         stream);
                compute_pressure_field();
            }
        } else {
            d2d(ut.p, u.p, U.npad);
            d2d(vt.p, v.p, V.npad);
            if (nw > 0) d2d(wt.p, w.p, W.npad);
            for (int sub = 0; sub < prm.N2; ++sub)
                pressure_step(false, u.p, v.p, w.p, ut.p, vt.p, wt.p, u.p, v.p, w.p);
        }
        Scalars after = s;
        divergence(after);
        s.MaxDeltaV = after.MaxDeltaV; s.normdiv = after.normdiv; s.velocityNorm = after.velocityNorm;
        s.maxdiv = after.maxdiv;
        if (method == NS3D_SIMPLERR) {
            res_row(it, s);
            relax_control(false);
            save_snapshot(it, savecounter);
        } else {
            save_snapshot(it, savecounter);
            relax_control(true);
        }
    }
    finish(name, it, s, t0, start);
}

// ============================ C-ABI =========================================
#define NS3D_TRY try {
#define NS3D_CATCH                                                   \
    }                                                                \
    catch (const ApiError &e) {                                      \
        return set_error(e.code, e.what());                          \
    }                                                                \
    catch (const CudaError &e) {                                     \
        return set_error(NS3D_ERR_CUDA, e.what());                   \
    }                                                                \
    catch (const std::bad_alloc &) {                                 \
        return set_error(NS3D_ERR_OOM, "host allocation failed");    \
    }                                                                \
    catch (const std::exception &e) {                                \
        return set_error(NS3D_ERR_ARG, e.what());                    \
    }

static ns3d_handle *checked(ns3d_handle *h) {
    if (!h) throw ApiError(NS3D_ERR_ARG, "NULL handle");
    return h;
}

// A NaN or an infinity in a host input would spread through every field of
// the solve (the reference accepts them); they are rejected at the boundary.
static void check_finite(const char *what, const double *x, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(x[i]))
            throw ApiError(NS3D_ERR_ARG, std::string(what) + ": value " + std::to_string(i) + " is not finite");
}

static void validate(const ns3d_params &p) {
    const struct {
        const char *name;
        double v;
    } reals[] = {{"dx", p.dx}, {"dy", p.dy}, {"dz", p.dz}, {"mu", p.mu}, {"rho", p.rho}, {"p0", p.p0},
                 {"gradp", p.gradp}, {"alpha", p.alpha}, {"beta", p.beta}, {"vsolvertol", p.vsolvertol},
                 {"psolvertol", p.psolvertol}, {"pcsolvertol", p.pcsolvertol}, {"simpletol", p.simpletol},
                 {"deltaRMR", p.deltaRMR}};
    for (const auto &r : reals)
        if (!std::isfinite(r.v)) throw ApiError(NS3D_ERR_ARG, std::string("parameter ") + r.name + " is not finite");
    if (p.dx <= 0 || p.mu <= 0 || p.rho <= 0) throw ApiError(NS3D_ERR_ARG, "dx, mu and rho must be > 0");
    if (p.maxitsolver <= 0 || p.maxitSIMPLE <= 0 || p.save_step <= 0)
        throw ApiError(NS3D_ERR_ARG, "maxitsolver, maxitSIMPLE and save_step must be > 0");
    if (p.direction < 1 || p.direction > 3) throw ApiError(NS3D_ERR_ARG, "direction must be 1, 2 or 3");
    if (p.border < 0) throw ApiError(NS3D_ERR_ARG, "border must be >= 0");
    if (p.method < NS3D_SIMPLEC || p.method > NS3D_IDEAL) throw ApiError(NS3D_ERR_ARG, "unknown method");
    if (p.precision != NS3D_FP64 && p.precision != NS3D_MIXED && p.precision != NS3D_MIXED_MG)
        throw ApiError(NS3D_ERR_ARG, "unknown precision");
    if (p.N1 < 0 || p.N2 < 0) throw ApiError(NS3D_ERR_ARG, "N1 and N2 must be >= 0");
}

extern "C" {

NS3D_API int ns3d_debug_barrier_timeout(int32_t extra_arrivals, double limit_s) {
    if (extra_arrivals < 0 || (extra_arrivals > 0 && !(limit_s > 0 && limit_s <= 10)))
        return set_error(NS3D_ERR_ARG, "ns3d_debug_barrier_timeout: extra_arrivals >= 0, 0 < limit_s <= 10");
    set_barrier_test((unsigned)extra_arrivals, extra_arrivals ? (unsigned long long)(limit_s * 1e9) : 0ull);
    return NS3D_OK;
}

NS3D_API int32_t ns3d_mixed_fallbacks(const ns3d_handle *h) { return h ? h->p_fallbacks : -1; }

NS3D_API int ns3d_abi_version(void) { return NS3D_ABI_VERSION; }
NS3D_API const char *ns3d_backend_name(void) { return "gb300"; }
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
    NS3D_TRY
    if (!params || !raw || !out) throw ApiError(NS3D_ERR_ARG, "ns3d_open: NULL argument");
    if (nx <= 0 || ny <= 0 || nz <= 0) throw ApiError(NS3D_ERR_ARG, "ns3d_open: bad image size");
    validate(*params);
    std::unique_ptr<ns3d_handle> H(new ns3d_handle());
    ns3d_handle &h = *H;
    h.prm = *params;
    if (h.prm.dy <= 0) h.prm.dy = h.prm.dx;
    if (h.prm.dz <= 0) h.prm.dz = h.prm.dx;
    if (h.prm.porevalue != 0 && h.prm.porevalue != 1) h.prm.porevalue = 0;
    NS3D_CUDA_CHECK(cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking));
    h.owned_stream.s = h.stream;
    h.build(raw, nx, ny, nz);
    h.dx = h.prm.dx; h.dy = h.prm.dy; h.dz = h.prm.dz; h.mu = h.prm.mu; h.rho = h.prm.rho;
    h.border = h.prm.border; h.deltaRMR = h.prm.deltaRMR;
    // constructor constants, src/NSBase.cxx:155-179
    h.set_pressure_drop(h.prm.p0, h.prm.gradp);
    h.mp.use_mg = h.prm.precision == NS3D_MIXED_MG;
    h.schemefactor = 0; h.min_alpha = 0.001; h.min_beta = 0.001; h.relax = 0.05;
    h.speedup = h.relax * 0.5; h.maxconvdelta = 2.5;
    h.alpha = h.alpha0 = h.prm.alpha;
    h.beta = h.beta0 = h.prm.beta;
    std::memset(&h.res, 0, sizeof h.res);
    h.default_fields();
    h.sync();
    *out = H.release();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_get_sizes(const ns3d_handle *h, ns3d_sizes *s) {
    if (!h || !s) return set_error(NS3D_ERR_ARG, "NULL argument");
    s->nx = h->nx; s->ny = h->ny; s->nz = h->nz;
    s->np = h->np; s->nu = h->nu; s->nv = h->nv; s->nw = h->nw; s->reserved = 0;
    return NS3D_OK;
}

NS3D_API int ns3d_get_index_arrays(ns3d_handle *H, int32_t *pi, int32_t *ui, int32_t *vi, int32_t *wi) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    if (pi) NS3D_CUDA_CHECK(cudaMemcpyAsync(pi, h.pmap.p, h.pmap.n * 4, cudaMemcpyDeviceToHost, h.stream));
    if (ui) NS3D_CUDA_CHECK(cudaMemcpyAsync(ui, h.umap.p, h.umap.n * 4, cudaMemcpyDeviceToHost, h.stream));
    if (vi) NS3D_CUDA_CHECK(cudaMemcpyAsync(vi, h.vmap.p, h.vmap.n * 4, cudaMemcpyDeviceToHost, h.stream));
    if (wi) NS3D_CUDA_CHECK(cudaMemcpyAsync(wi, h.wmap.p, h.wmap.n * 4, cudaMemcpyDeviceToHost, h.stream));
    h.sync();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_set_initial_fields(ns3d_handle *H, const double *pimg, const double *uimg, const double *vimg,
                                     const double *wimg) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    const long N = (long)h.nx * h.ny * h.nz, NU = (long)(h.nx + 1) * h.ny * h.nz;
    if (pimg) check_finite("initial pressure field", pimg, (size_t)N);
    if (uimg) check_finite("initial x velocity field", uimg, (size_t)NU);
    if (vimg) check_finite("initial y velocity field", vimg, (size_t)N);
    if (wimg) check_finite("initial z velocity field", wimg, (size_t)N);
    h.default_fields();
    DBuf<double> tmp;
    tmp.alloc((size_t)NU, h.stream);
    auto put = [&](const double *src, const int *map, long cells, double *f) {
        if (!src) return;
        NS3D_CUDA_CHECK(cudaMemcpyAsync(tmp.p, src, cells * 8, cudaMemcpyHostToDevice, h.stream));
        launch_scatter_image(map, cells, tmp.p, f, h.stream);
        h.sync();
    };
    put(pimg, h.pmap.p, N, h.p.p);
    put(uimg, h.umap.p, NU, h.u.p);
    put(vimg, h.vmap.p, N, h.v.p);
    put(wimg, h.wmap.p, N, h.w.p);
    h.sync();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_get_fields(ns3d_handle *H, double *p, double *u, double *v, double *w) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    if (p) NS3D_CUDA_CHECK(cudaMemcpyAsync(p, h.p.p, (size_t)h.np * 8, cudaMemcpyDeviceToHost, h.stream));
    if (u) NS3D_CUDA_CHECK(cudaMemcpyAsync(u, h.u.p, (size_t)h.nu * 8, cudaMemcpyDeviceToHost, h.stream));
    if (v) NS3D_CUDA_CHECK(cudaMemcpyAsync(v, h.v.p, (size_t)h.nv * 8, cudaMemcpyDeviceToHost, h.stream));
    if (w) NS3D_CUDA_CHECK(cudaMemcpyAsync(w, h.w.p, (size_t)h.nw * 8, cudaMemcpyDeviceToHost, h.stream));
    h.sync();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_set_fields(ns3d_handle *H, const double *p, const double *u, const double *v, const double *w) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    if (p) check_finite("pressure field", p, (size_t)h.np);
    if (u) check_finite("x velocity field", u, (size_t)h.nu);
    if (v) check_finite("y velocity field", v, (size_t)h.nv);
    if (w) check_finite("z velocity field", w, (size_t)h.nw);
    if (p) NS3D_CUDA_CHECK(cudaMemcpyAsync(h.p.p, p, (size_t)h.np * 8, cudaMemcpyHostToDevice, h.stream));
    if (u) NS3D_CUDA_CHECK(cudaMemcpyAsync(h.u.p, u, (size_t)h.nu * 8, cudaMemcpyHostToDevice, h.stream));
    if (v) NS3D_CUDA_CHECK(cudaMemcpyAsync(h.v.p, v, (size_t)h.nv * 8, cudaMemcpyHostToDevice, h.stream));
    if (w) NS3D_CUDA_CHECK(cudaMemcpyAsync(h.w.p, w, (size_t)h.nw * 8, cudaMemcpyHostToDevice, h.stream));
    h.sync();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_get_field_images(ns3d_handle *H, double *pimg, double *uimg, double *vimg, double *wimg,
                                   double *vavg) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    const long N = (long)h.nx * h.ny * h.nz, NU = (long)(h.nx + 1) * h.ny * h.nz;
    DBuf<double> tmp;
    tmp.alloc((size_t)std::max(3 * N, NU), h.stream);
    auto get = [&](double *dst, const int *map, long cells, const double *f) {
        if (!dst) return;
        launch_gather_image(map, cells, f, tmp.p, h.stream);
        NS3D_CUDA_CHECK(cudaMemcpyAsync(dst, tmp.p, cells * 8, cudaMemcpyDeviceToHost, h.stream));
        h.sync();
    };
    get(pimg, h.pmap.p, N, h.p.p);
    get(uimg, h.umap.p, NU, h.u.p);
    get(vimg, h.vmap.p, N, h.v.p);
    get(wimg, h.wmap.p, N, h.w.p);
    if (vavg) {
        launch_face_average(h.grid(), h.u.p, h.v.p, h.w.p, tmp.p, h.stream);
        NS3D_CUDA_CHECK(cudaMemcpyAsync(vavg, tmp.p, 3 * N * 8, cudaMemcpyDeviceToHost, h.stream));
        h.sync();
    }
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_set_output(ns3d_handle *H, const char *dir, const char *stem, int32_t write_fields) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    h.info.close();
    h.resl.close();
    h.have_out = false;
    if (!dir) return NS3D_OK;
    h.outdir = dir;
    h.stem = stem ? stem : "image";
    h.write_fields = write_fields != 0;
    std::string d = h.outdir.empty() ? std::string() : h.outdir + "/";
    std::string tag = std::to_string(h.prm.direction) + "-" + h.stem;
    if (!h.info.open(d + "INFO-" + tag + ".log", 15) || !h.resl.open(d + "RES-" + tag + ".csv", 6))
        throw ApiError(NS3D_ERR_IO, std::string("cannot open log files in ") + dir);
    h.have_out = true;
    // the constructor lines that reach the INFO file, src/NSBase.cxx:143,182-187
    h.info.s("Size ").i(h.nx).s(",").i(h.ny).s(",").i(h.nz).nl();
    h.info.s("Porosity: ").d((double)(float(h.np) / float((long)h.nx * h.ny * h.nz))).nl();
    h.info.s("Nodes for the pressure field: ").i(h.np).nl();
    h.info.s("Nodes for the u velocity field: ").i(h.nu).nl();
    h.info.s("Nodes for the v velocity field: ").i(h.nv).nl();
    h.info.s("Nodes for the w velocity field: ").i(h.nw).nl();
    h.info.s("Delta RMR min : ").d(h.deltaRMR).nl();
    return NS3D_OK;
    NS3D_CATCH
}

// the state a solve starts from: no result, initial relaxation, no history
void ns3d_handle::begin_solve() {
    std::memset(&res, 0, sizeof res);
    p_fp64 = false;
    p_fallbacks = 0;
    su = sv = sw = sp = SolveOutcome();
    alpha = alpha0;
    beta = beta0;
    avgRMR.clear();
    RMR = old_RMR = 0;
    kmom.reset_launch_count();
    kp.reset_launch_count();
}

NS3D_API int ns3d_solve(ns3d_handle *H) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    h.begin_solve();
    // while several solves run at once the loop kernels take fewer SMs each
    ActiveSolve active;
    struct Member {  // a merged solve counts as a member of its group while it runs
        SolveGroup *g;
        explicit Member(SolveGroup *grp) : g(grp) {
            if (g) g->join();
        }
        ~Member() {
            if (g) g->leave();
        }
    } member(h.group);
    if (h.prm.method == NS3D_SIMPLEC) h.run_simplec();
    else h.run_simpler_family(h.prm.method);
    return NS3D_OK;
    NS3D_CATCH
}

static int solve_lockstep(ns3d_handle *const *hs, int32_t n, int32_t *status) {
    NS3D_TRY
    if (n < 0 || (n > 0 && !hs)) throw ApiError(NS3D_ERR_ARG, "ns3d_solve_lockstep: bad arguments");
    for (int i = 0; i < n; ++i) {
        checked(hs[i]);
        for (int j = 0; j < i; ++j)
            if (hs[j] == hs[i]) throw ApiError(NS3D_ERR_ARG, "ns3d_solve_lockstep: a handle appears twice");
    }
    if (n == 0) return NS3D_OK;
    return lockstep_solve(hs, n, status);
    NS3D_CATCH
}

NS3D_API int ns3d_solve_lockstep(ns3d_handle *const *hs, int32_t n, int32_t *status) {
    const int rc = solve_lockstep(hs, n, status);
    if (rc != NS3D_OK && status)
        for (int i = 0; i < n; ++i) status[i] = rc;
    return rc;
}

NS3D_API int ns3d_batch_solve_lockstep(const ns3d_params *params, const uint8_t *const *raws, const int32_t *dims,
                                       int32_t n, ns3d_result *results, int32_t *status) {
    if (!params || !raws || !dims || !results || n < 0) return set_error(NS3D_ERR_ARG, "bad batch arguments");
    std::vector<ns3d_handle *> hs;
    std::vector<int> idx;
    int worst = NS3D_OK;
    for (int i = 0; i < n; ++i) {
        std::memset(&results[i], 0, sizeof results[i]);
        ns3d_handle *h = nullptr;
        const int rc = ns3d_open(&params[i], raws[i], dims[3 * i], dims[3 * i + 1], dims[3 * i + 2], &h);
        if (status) status[i] = rc;
        if (rc != NS3D_OK) {
            worst = rc;
            continue;
        }
        hs.push_back(h);
        idx.push_back(i);
    }
    std::vector<int32_t> st(hs.size(), NS3D_OK);
    const int rc = ns3d_solve_lockstep(hs.data(), (int32_t)hs.size(), st.data());
    if (rc != NS3D_OK) worst = rc;
    for (size_t k = 0; k < hs.size(); ++k) {
        if (status) status[idx[k]] = st[k];
        if (st[k] == NS3D_OK) ns3d_get_result(hs[k], &results[idx[k]]);
        ns3d_close(hs[k]);
    }
    return worst;
}

NS3D_API int ns3d_solve_sweep(ns3d_handle *H, const double *gradp, int32_t n, int32_t warm_start,
                              ns3d_result *results) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    if (n < 0 || (n > 0 && (!gradp || !results))) throw ApiError(NS3D_ERR_ARG, "bad sweep arguments");
    const double p0_user = h.prm.p0;
    for (int i = 0; i < n; ++i) {
        const double old_p0 = h.p0, old_gradp = h.gradp;
        h.prm.gradp = gradp[i];
        h.set_pressure_drop(p0_user, gradp[i]);
        if (!warm_start || i == 0 || old_gradp == 0.0) {
            h.default_fields();
        } else {
            // Stokes flow is linear in the pressure drop: scale the previous solution
            const double ratio = gradp[i] / old_gradp;
            launch_scale_fields(h.u.p, h.U.npad, h.v.p, h.V.npad, h.w.p, h.W.npad, h.p.p, h.P.npad, ratio, old_p0,
                                h.p0, h.stream);
            NS3D_CUDA_CHECK(cudaMemsetAsync(h.pc.p, 0, h.pc.n * 8, h.stream));
        }
        const int rc = ns3d_solve(H);
        if (rc != NS3D_OK) return rc;
        results[i] = h.res;
    }
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_set_group(ns3d_handle *H, ns3d_group *g) {
    NS3D_TRY
    checked(H)->group = group_of(g);
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_get_result(const ns3d_handle *h, ns3d_result *r) {
    if (!h || !r) return set_error(NS3D_ERR_ARG, "NULL argument");
    *r = h->res;
    return NS3D_OK;
}

NS3D_API int ns3d_assemble_momentum(ns3d_handle *H) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    h.assemble_all_momentum();
    h.momentum_rhs();
    h.sync();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_assemble_pressure_correction(ns3d_handle *H, int32_t simplec) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    launch_assemble_pressure(simplec ? 1 : 2, 0, h.grid(), h.phys(), h.P.view(), h.U.view(), h.V.view(), h.W.view(),
                             h.u.p, h.v.p, h.w.p, h.p.p, h.stream);
    h.sync();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_assemble_pressure(ns3d_handle *H, int32_t relax) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    h.hats(h.u.p, h.v.p, h.w.p, h.u.p, h.v.p, h.w.p);
    launch_assemble_pressure(0, relax ? 1 : 0, h.grid(), h.phys(), h.P.view(), h.U.view(), h.V.view(), h.W.view(),
                             h.uh.p, h.vh.p, h.wh.p, h.p.p, h.stream);
    h.sync();
    return NS3D_OK;
    NS3D_CATCH
}

static DevSys *sys_of(ns3d_handle &h, int sys) {
    switch (sys) {
        case NS3D_SYS_U: return &h.U;
        case NS3D_SYS_V: return &h.V;
        case NS3D_SYS_W: return &h.W;
        case NS3D_SYS_P: return &h.P;
        default: throw ApiError(NS3D_ERR_ARG, "bad system index");
    }
}

NS3D_API int ns3d_get_system(ns3d_handle *H, int32_t sys, double *coef, int32_t *nbr, double *rhs, double *rowsum) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    DevSys &S = *sys_of(h, sys);
    const size_t n = (size_t)S.n;
    for (int s = 0; s < 7 && coef; ++s)
        NS3D_CUDA_CHECK(cudaMemcpyAsync(coef + s * n, S.coef.p + (size_t)s * S.npad, n * 8, cudaMemcpyDeviceToHost,
                                        h.stream));
    for (int s = 0; s < 6 && nbr; ++s)
        NS3D_CUDA_CHECK(cudaMemcpyAsync(nbr + s * n, S.nbr.p + (size_t)s * S.npad, n * 4, cudaMemcpyDeviceToHost,
                                        h.stream));
    if (rhs) NS3D_CUDA_CHECK(cudaMemcpyAsync(rhs, S.rhs.p, n * 8, cudaMemcpyDeviceToHost, h.stream));
    if (rowsum) NS3D_CUDA_CHECK(cudaMemcpyAsync(rowsum, S.rowsum.p, n * 8, cudaMemcpyDeviceToHost, h.stream));
    h.sync();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_solve_system(ns3d_handle *H, int32_t sys, const double *rhs, double *x, double tol, int32_t maxit,
                               ns3d_solve_info *info) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    if (!x || maxit <= 0) throw ApiError(NS3D_ERR_ARG, "ns3d_solve_system: bad argument");
    DevSys &S = *sys_of(h, sys);
    DBuf<double> dx, db;
    dx.alloc_zero(S.npad, h.stream);
    NS3D_CUDA_CHECK(cudaMemcpyAsync(dx.p, x, (size_t)S.n * 8, cudaMemcpyHostToDevice, h.stream));
    const double *b = S.rhs.p;
    if (rhs) {
        db.alloc_zero(S.npad, h.stream);
        NS3D_CUDA_CHECK(cudaMemcpyAsync(db.p, rhs, (size_t)S.n * 8, cudaMemcpyHostToDevice, h.stream));
        b = db.p;
    }
    std::vector<SolveOutcome> out;
    if (h.mixed()) {
        MixedSet ms;
        ms.use_mg = h.prm.precision == NS3D_MIXED_MG;  // pressure systems (cell extents known) only
        ms.run({{&S, dx.p, b, tol, maxit}}, h.stream, out);
    } else {
        KrylovSet ks;
        ks.run({{&S, dx.p, b, tol, maxit}}, h.stream, out);
    }
    NS3D_CUDA_CHECK(cudaMemcpyAsync(x, dx.p, (size_t)S.n * 8, cudaMemcpyDeviceToHost, h.stream));
    h.sync();
    if (info) {
        info->iterations = out[0].iters;
        info->info = out[0].info;
        info->error = out[0].error;
    }
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_close(ns3d_handle *h) {
    delete h;
    return NS3D_OK;
}

static int64_t g_launch_base = 0;

NS3D_API int64_t ns3d_kernel_launches(void) { return launch_count(); }

NS3D_API int ns3d_set_profiling(ns3d_handle *H, int32_t enable) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    h.kp.profiling = enable != 0;
    h.kp.prof = KrylovSet::Profile();
    g_launch_base = launch_count();
    return NS3D_OK;
    NS3D_CATCH
}

NS3D_API int ns3d_get_profile(ns3d_handle *H, ns3d_profile *out) {
    NS3D_TRY
    ns3d_handle &h = *checked(H);
    if (!out) throw ApiError(NS3D_ERR_ARG, "NULL profile");
    for (int k = 0; k < 6; ++k) {
        out->launches[k] = h.kp.prof.launches[k];
        out->ms[k] = h.kp.prof.ms[k];
        out->rows[k] = h.kp.prof.rows[k];
    }
    out->total_launches = launch_count() - g_launch_base;
    return NS3D_OK;
    NS3D_CATCH
}

}  // extern "C"
