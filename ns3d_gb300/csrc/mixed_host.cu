// mixed_host.cu -- host driver of the mixed-precision solves (see mixed.cu).
#include <algorithm>
#include <cstring>

#include "mixed.h"
#include "runtime.h"
#include "tuner.h"

namespace ns3d {

void DevSys::allocate_f32(cudaStream_t st) {
    if (coef32.n) return;
    coef32.alloc_zero((size_t)7 * npad, st);
    invdiag32.alloc_zero(npad, st);
    for (DBuf<float> *b : {&fx, &fr, &fr0, &fp, &fv, &fy, &fs, &fz, &ft, &fp2, &fv2}) b->alloc_zero(npad, st);
}

// The aggregation hierarchy of system S from its cells: level k+1 groups
// the rows of level k by the 2x2x2 block of their cell coordinates, until
// a level has at most kMGCoarsest rows or MG_MAX levels exist.
constexpr int kMGCoarsest = 512;

static void build_mg(DevSys &S, cudaStream_t st) {
    std::vector<int> cell((size_t)S.n);
    NS3D_CUDA_CHECK(cudaMemcpyAsync(cell.data(), S.cell.p, (size_t)S.n * 4, cudaMemcpyDeviceToHost, st));
    NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
    std::vector<long long> ci(S.n), cj(S.n), ck(S.n);
    for (int r = 0; r < S.n; ++r) {
        const long long c = cell[r];
        ck[r] = c % S.cell_nz;
        cj[r] = (c / S.cell_nz) % S.cell_ny;
        ci[r] = c / ((long long)S.cell_nz * S.cell_ny);
    }
    std::unique_ptr<MGHost> H(new MGHost());
    int nf = S.n;
    while (H->nlev < MG_MAX && nf > kMGCoarsest) {
        // blocks of the current rows, numbered in ascending key order
        std::vector<std::pair<long long, int>> key(nf);
        for (int r = 0; r < nf; ++r) key[r] = {((ci[r] >> 1) << 42) | ((cj[r] >> 1) << 21) | (ck[r] >> 1), r};
        std::sort(key.begin(), key.end());
        std::vector<int> agg(nf);
        std::vector<long long> bkey;
        for (int q = 0; q < nf; ++q) {
            if (q == 0 || key[q].first != key[q - 1].first) bkey.push_back(key[q].first);
            agg[key[q].second] = (int)bkey.size() - 1;
        }
        const int nc = (int)bkey.size();
        std::vector<int> mstart(nc + 1, 0), members(nf);
        for (int r = 0; r < nf; ++r) mstart[agg[r] + 1]++;
        for (int I = 0; I < nc; ++I) mstart[I + 1] += mstart[I];
        std::vector<int> fill(mstart.begin(), mstart.end() - 1);
        for (int r = 0; r < nf; ++r) members[fill[agg[r]]++] = r;  // ascending rows within a block
        const int npad = (nc + 255) / 256 * 256;
        std::vector<int> nbr((size_t)6 * npad, -1);
        std::vector<long long> ni(nc), nj(nc), nk(nc);
        for (int I = 0; I < nc; ++I) {
            ni[I] = bkey[I] >> 42;
            nj[I] = (bkey[I] >> 21) & ((1LL << 21) - 1);
            nk[I] = bkey[I] & ((1LL << 21) - 1);
        }
        auto find = [&](long long a, long long b, long long c) -> int {
            if (a < 0 || b < 0 || c < 0) return -1;
            const long long k = (a << 42) | (b << 21) | c;
            auto it = std::lower_bound(bkey.begin(), bkey.end(), k);
            return (it != bkey.end() && *it == k) ? (int)(it - bkey.begin()) : -1;
        };
        for (int I = 0; I < nc; ++I) {  // directions W, E, S, N, B, T
            nbr[(size_t)0 * npad + I] = find(ni[I] - 1, nj[I], nk[I]);
            nbr[(size_t)1 * npad + I] = find(ni[I] + 1, nj[I], nk[I]);
            nbr[(size_t)2 * npad + I] = find(ni[I], nj[I] - 1, nk[I]);
            nbr[(size_t)3 * npad + I] = find(ni[I], nj[I] + 1, nk[I]);
            nbr[(size_t)4 * npad + I] = find(ni[I], nj[I], nk[I] - 1);
            nbr[(size_t)5 * npad + I] = find(ni[I], nj[I], nk[I] + 1);
        }
        MGHostLevel &L = H->lev[++H->nlev];
        L.n = nc;
        L.npad = npad;
        L.nbr.alloc(nbr.size(), st);
        L.agg.alloc(agg.size(), st);
        L.mstart.alloc(mstart.size(), st);
        L.members.alloc(members.size(), st);
        NS3D_CUDA_CHECK(cudaMemcpyAsync(L.nbr.p, nbr.data(), nbr.size() * 4, cudaMemcpyHostToDevice, st));
        NS3D_CUDA_CHECK(cudaMemcpyAsync(L.agg.p, agg.data(), agg.size() * 4, cudaMemcpyHostToDevice, st));
        NS3D_CUDA_CHECK(cudaMemcpyAsync(L.mstart.p, mstart.data(), mstart.size() * 4, cudaMemcpyHostToDevice, st));
        NS3D_CUDA_CHECK(cudaMemcpyAsync(L.members.p, members.data(), members.size() * 4, cudaMemcpyHostToDevice, st));
        L.coef.alloc_zero((size_t)7 * npad, st);
        for (DBuf<float> *b : {&L.invdiag, &L.x, &L.b, &L.t}) b->alloc_zero(npad, st);
        NS3D_CUDA_CHECK(cudaStreamSynchronize(st));  // the host vectors above are temporaries
        ci = std::move(ni);
        cj = std::move(nj);
        ck = std::move(nk);
        nf = nc;
    }
    S.mg = std::move(H);
}

template <int CAP>
void MixedSetT<CAP>::configure(const std::vector<SolveItem> &items, cudaStream_t st) {
    std::vector<const double *> key;
    for (const SolveItem &it : items) {
        key.push_back(it.sys->coef.p);
        key.push_back(it.x);
        key.push_back(it.b);
    }
    // a merged set's members come and go (a new solve may reuse a finished
    // one's addresses): it is set up afresh every run
    if (CAP <= KMAX && key == key_) return;
    const int ns = (int)items.size();
    if (ns > CAP) throw ApiError(NS3D_ERR_ARG, "too many systems in one solve set");
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
        // a solver instance's own set: the multilevel preconditioner for a
        // single system; a merged set: what each system's own set chose
        const bool mg = CAP > KMAX ? (items[i].mg && S.mg)
                                   : (use_mg && ns == 1 && S.n > kMGCoarsest && S.cell_ny > 0);
        if (mg) {
            if (!S.mg) build_mg(S, st);
            m.mg.nlev = S.mg->nlev;
            m.mg.sweeps = 30;
            m.mg.omega = 0.6f;
            for (int k = 1; k <= S.mg->nlev; ++k) {
                MGHostLevel &H = S.mg->lev[k];
                MGLevel &G = m.mg.lev[k];
                G.n = H.n;
                G.npad = H.npad;
                G.nbr = H.nbr.p;
                G.coef = H.coef.p;
                G.invdiag = H.invdiag.p;
                G.agg = H.agg.p;
                G.mstart = H.mstart.p;
                G.members = H.members.p;
                G.x = H.x.p;
                G.b = H.b.p;
                G.t = H.t.p;
            }
        }
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

template <int CAP>
int MixedSetT<CAP>::variant() const {
    long rows = 0;
    bool mg = false;
    for (int i = 0; i < nsys_; ++i) {
        rows += set_.sys[i].n;
        mg = mg || set_.sys[i].mg.nlev > 0;
    }
    return m32_fused(rows, mg) ? 1 : 0;
}

template <int CAP>
void MixedSetT<CAP>::run(const std::vector<SolveItem> &items, cudaStream_t st, std::vector<SolveOutcome> &out,
                         int variant) {
    configure(items, st);
    const int ns = nsys_;
    int maxit = 0;
    for (int i = 0; i < ns; ++i) {
        DevSys &S = *items[i].sys;
        launch_to_f32(S.coef.p, S.invdiag.p, S.npad, S.coef32.p, S.invdiag32.p, st);
        if (set_.sys[i].mg.nlev > 0) launch_mg_galerkin(set_.sys[i], st);
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
    // merged sets: the grid of each FP32 loop launch comes from the
    // autotuner, told the launch's time per inner row-iteration
    const bool tune = CAP > KMAX;
    int cand = 0, kind = 0;
    if (tune) {
        bool mg = false;
        for (int i = 0; i < ns; ++i) mg = mg || set_.sys[i].mg.nlev > 0;
        kind = mg ? 3 : (variant == 1 ? 2 : 1);
        if (!ev_[0])
            for (cudaEvent_t &e : ev_) NS3D_CUDA_CHECK(cudaEventCreate(&e));
    }
    const uint64_t tkey = tuner_key(kind, (long)total_chunks_ * MSUB, share);
    std::vector<int> iters_before(ns, 0);
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
        if (tune && rounds > 0) {  // inner iterations of the round, from the FP64 states
            double rows = 0;
            for (int i = 0; i < ns; ++i) rows += (double)set_.sys[i].n * (h_dc_.p[i].total_iter - iters_before[i]);
            float ms = 0;
            NS3D_CUDA_CHECK(cudaEventElapsedTime(&ms, ev_[0], ev_[1]));
            grid_tuner().report(tkey, cand, ms, rows);
        }
        for (int i = 0; i < ns; ++i) iters_before[i] = h_dc_.p[i].total_iter;
        bool all_done = true;
        for (int i = 0; i < ns; ++i) all_done = all_done && h_dc_.p[i].done;
        if (all_done) break;
        if (++rounds > maxit + 2L) throw ApiError(NS3D_ERR_TIMEOUT, "defect correction exceeded its round bound");
        launch_m32_init(set_, st);
        if (tune) {
            cand = grid_tuner().choose(tkey);
            NS3D_CUDA_CHECK(cudaEventRecord(ev_[0], st));
        }
        NS3D_CUDA_CHECK(launch_m32_loop(set_, bar_.p, maxit + 64, st, variant, share << cand));
        if (tune) NS3D_CUDA_CHECK(cudaEventRecord(ev_[1], st));
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

template <int CAP>
MixedSetT<CAP>::~MixedSetT() {
    for (cudaEvent_t e : ev_)
        if (e) cudaEventDestroy(e);
}

template class MixedSetT<KMAX>;
template class MixedSetT<KMAX_MERGED_M>;

}  // namespace ns3d
