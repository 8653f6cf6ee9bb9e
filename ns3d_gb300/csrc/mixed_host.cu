// mixed_host.cu -- host driver of the mixed-precision solves (see mixed.cu).
#include <cstring>

#include "mixed.h"
#include "runtime.h"

namespace ns3d {

void DevSys::allocate_f32(cudaStream_t st) {
    if (coef32.n) return;
    coef32.alloc_zero((size_t)7 * npad, st);
    invdiag32.alloc_zero(npad, st);
    for (DBuf<float> *b : {&fx, &fr, &fr0, &fp, &fv, &fy, &fs, &fz, &ft, &fp2, &fv2}) b->alloc_zero(npad, st);
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
    if (!bar_.n) {
        bar_.alloc_zero(1, st);
        h_err_.alloc(1);
    }
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
        m.p2 = S.fp2.p; m.v2 = S.fv2.p;
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
        d.inner_cap = inner_cap;
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
    // One round = FP32 init, the FP32 loop kernel (it ends when every inner
    // solve of the round is done: each is capped by the remaining iteration
    // budget), the FP64 update and residual; the host reads the outer state
    // once per round.
    while (true) {
        NS3D_CUDA_CHECK(cudaMemcpyAsync(h_dc_.p, dc_.p, ns * sizeof(DCState), cudaMemcpyDeviceToHost, st));
        NS3D_CUDA_CHECK(cudaMemcpyAsync(h_err_.p, &bar_.p->err, sizeof(int), cudaMemcpyDeviceToHost, st));
        NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
        if (rounds > 0 && h_err_.p[0])
            throw ApiError(NS3D_ERR_TIMEOUT, "FP32 BiCGSTAB loop kernel: a grid barrier timed out");
        bool all_done = true;
        for (int i = 0; i < ns; ++i) all_done = all_done && h_dc_.p[i].done;
        if (all_done) break;
        if (++rounds > maxit + 2L) throw ApiError(NS3D_ERR_TIMEOUT, "defect correction exceeded its round bound");
        launch_m32_init(set_, st);
        NS3D_CUDA_CHECK(launch_m32_loop(set_, bar_.p, maxit + 64, st));
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
    }
    NS3D_CUDA_CHECK(cudaMemcpyAsync(out_st_.p, h_out_.p, ns * sizeof(KState), cudaMemcpyHostToDevice, st));
}

}  // namespace ns3d
