// mixed_host.cu -- host driver of the mixed-precision solves (see mixed.cu).
#include <cstring>

#include "mixed.h"
#include "runtime.h"

namespace ns3d {

void DevSys::allocate_f32(cudaStream_t st) {
    if (coef32.n) return;
    coef32.alloc_zero((size_t)7 * npad, st);
    invdiag32.alloc_zero(npad, st);
    for (DBuf<float> *b : {&fx, &fr, &fr0, &fp, &fv, &fy, &fs, &fz, &ft}) b->alloc_zero(npad, st);
}

void MixedSet::configure(const std::vector<SolveItem> &items, cudaStream_t st) {
    std::vector<const double *> key;
    for (const SolveItem &it : items) {
        key.push_back(it.sys->coef.p);
        key.push_back(it.x);
        key.push_back(it.b);
    }
    if (key == key_) return;
    const int ns = (int)items.size();
    if (ns > KMAX) throw ApiError(NS3D_ERR_ARG, "too many systems in one solve set");
    std::vector<MSys> ms(ns);
    int chunk = 0;
    if ((int)st_.n < ns) {
        st_.alloc_zero(ns, st);
        out_st_.alloc_zero(ns, st);
        dc_.alloc_zero(ns, st);
        h_st_.alloc(ns);
        h_out_.alloc(ns);
        h_dc_.alloc(ns);
    }
    for (int i = 0; i < ns; ++i) {
        DevSys &S = *items[i].sys;
        S.allocate_f32(st);
        MSys &m = ms[i];
        std::memset(&m, 0, sizeof m);
        m.n = S.n;
        m.npad = S.npad;
        m.nchunks = S.nchunks;
        m.chunk_begin = chunk;
        chunk += S.nchunks;
        m.nbr = S.nbr.p;
        m.coef64 = S.coef.p;
        m.b64 = items[i].b;
        m.x64 = items[i].x;
        m.r64 = S.r.p;
        m.coef32 = S.coef32.p;
        m.invdiag32 = S.invdiag32.p;
        m.x = S.fx.p; m.r = S.fr.p; m.r0 = S.fr0.p; m.p = S.fp.p; m.v = S.fv.p;
        m.y = S.fy.p; m.s = S.fs.p; m.z = S.fz.p; m.t = S.ft.p;
        m.part = S.part.p;
        m.st = st_.p + i;
        m.dc = dc_.p + i;
    }
    std::memset(&set_, 0, sizeof set_);
    set_.nsys = ns;
    set_.total_chunks = chunk;
    for (int i = 0; i < ns; ++i) set_.sys[i] = ms[i];
    NS3D_CUDA_CHECK(cudaStreamSynchronize(st));  // FP32 buffers allocated above
    key_ = key;
    nsys_ = ns;
    total_chunks_ = chunk;
}

void MixedSet::run(const std::vector<SolveItem> &items, cudaStream_t st, std::vector<SolveOutcome> &out) {
    configure(items, st);
    const int ns = nsys_;
    int maxit = 0;
    for (int i = 0; i < ns; ++i) {
        DevSys &S = *items[i].sys;
        launch_to_f32(S.coef.p, S.invdiag.p, S.npad, S.coef32.p, S.invdiag32.p, st);
        DCState d;
        std::memset(&d, 0, sizeof d);
        d.tol = items[i].tol;
        d.maxit = items[i].maxit;
        d.tin_min = inner_rel_tol;
        if (S.n == 0) {
            d.done = 1;
            d.zero_rhs = 1;
            d.total_iter = d.maxit;
            d.error = d.tol;
        }
        h_dc_.p[i] = d;
        KState k;
        std::memset(&k, 0, sizeof k);
        h_st_.p[i] = k;
        maxit = std::max(maxit, items[i].maxit);
    }
    NS3D_CUDA_CHECK(cudaMemcpyAsync(dc_.p, h_dc_.p, ns * sizeof(DCState), cudaMemcpyHostToDevice, st));
    NS3D_CUDA_CHECK(cudaMemcpyAsync(st_.p, h_st_.p, ns * sizeof(KState), cudaMemcpyHostToDevice, st));
    launch_dc_resid(set_, 1, st);
    // Every round runs at least one inner iteration per unfinished system, so
    // maxit + 2 rounds bound the loop; each round's inner loop is bounded by
    // the remaining iteration budget.
    long rounds = 0;
    int work_total = 0;
    std::vector<int> work(ns, 0);
    while (true) {
        NS3D_CUDA_CHECK(cudaMemcpyAsync(h_dc_.p, dc_.p, ns * sizeof(DCState), cudaMemcpyDeviceToHost, st));
        NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
        bool all_done = true;
        for (int i = 0; i < ns; ++i) all_done = all_done && h_dc_.p[i].done;
        if (all_done) break;
        if (++rounds > maxit + 2L) throw ApiError(NS3D_ERR_TIMEOUT, "defect correction exceeded its round bound");
        launch_m32_init(set_, st);
        long issued = 0;
        int batch = std::max(1, std::min(32, prev_iters_ / 2));
        while (true) {
            for (int b = 0; b < batch; ++b) launch_m32_iteration(set_, st);
            issued += batch;
            batch = std::min(64, batch * 2);
            NS3D_CUDA_CHECK(cudaMemcpyAsync(h_st_.p, st_.p, ns * sizeof(KState), cudaMemcpyDeviceToHost, st));
            NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
            bool inner_done = true;
            for (int i = 0; i < ns; ++i)
                if (!h_dc_.p[i].done && !h_st_.p[i].done) inner_done = false;
            if (inner_done) break;
            if (issued > maxit + 64L) throw ApiError(NS3D_ERR_TIMEOUT, "FP32 BiCGSTAB exceeded its iteration bound");
        }
        int round_max = 0;
        for (int i = 0; i < ns; ++i)
            if (!h_dc_.p[i].done) round_max = std::max(round_max, h_st_.p[i].iter);
        prev_iters_ = std::max(2, round_max);
        launch_dc_update(set_, st);
        launch_dc_resid(set_, 0, st);
    }
    NS3D_CUDA_CHECK(cudaMemcpyAsync(h_st_.p, st_.p, ns * sizeof(KState), cudaMemcpyDeviceToHost, st));
    NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
    out.assign(ns, SolveOutcome());
    for (int i = 0; i < ns; ++i) {
        const DCState &d = h_dc_.p[i];
        out[i].iters = d.total_iter;
        out[i].info = d.info;
        out[i].error = d.error;
        out[i].work = h_st_.p[i].work;
        out[i].valid = true;
        KState k;
        std::memset(&k, 0, sizeof k);
        k.iter = d.total_iter;
        k.info = d.info;
        k.done = 1;
        h_out_.p[i] = k;
        work_total += out[i].work;
    }
    (void)work_total;
    NS3D_CUDA_CHECK(cudaMemcpyAsync(out_st_.p, h_out_.p, ns * sizeof(KState), cudaMemcpyHostToDevice, st));
}

}  // namespace ns3d
