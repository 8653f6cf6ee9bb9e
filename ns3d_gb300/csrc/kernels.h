// kernels.h -- host-side launchers of the NS3D device kernels.
#pragma once

#include <algorithm>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ns3d {

struct Grid;
struct SysView;
struct KSys;
template <int CAP>
struct KSetArgT;
struct GridBar;
struct LoopProf;
struct KState;

// geometry.cu
void launch_build_image(const uint8_t *raw, int rnx, int rny, int rnz, int dir, int border, int pv, uint8_t *img,
                        int nx, int ny, int nz, cudaStream_t st);
int index_build_blocks(long ncells);
void launch_index_build(const uint8_t *img, int nx, int ny, int nz, int4 *blk, int4 *totals, int *pmap, int *umap,
                        int *vmap, int *wmap, int *pcell, int *ucell, int *vcell, int *wcell, cudaStream_t st);
void launch_nbr_mom(const int *map, int d0, int ny, int nz, const int *cell, int n, int npad, int *nbr, int zdir,
                    cudaStream_t st);
void launch_nbr_p(const Grid &g, const int *cell, int n, int npad, int *nbr, cudaStream_t st);

// physics.cu: assembly, corrections, diagnostics
struct Phys {
    double dx, dy, dz, mu, rho, alpha, beta, p0, p1, schemefactor;
    // 1/dx, 1/dy, 1/dz, 1/dx^2, 1/dy^2, 1/dz^2 computed once on the host
    // (IEEE division is correctly rounded: the same bits as in the kernels)
    double idx, idy, idz, idx2, idy2, idz2;
};
// momentum systems: coefficients, row sums and Jacobi inverse diagonal
void launch_assemble_momentum(int comp, const Grid &g, const Phys &ph, const SysView &A, const double *uc,
                              const double *vc, const double *wc, cudaStream_t st);
// momentum right-hand sides (comp 0,1,2)
void launch_momentum_rhs(int comp, const Grid &g, const Phys &ph, const SysView &A, const double *p,
                         const double *x, cudaStream_t st);
// pseudo-velocities x_hat = -(sum a_nb x_c[nb]) / a_P + x_old (1-alpha)
void launch_hat(const SysView &A, const Phys &ph, const double *xc, const double *xold, double *hat,
                cudaStream_t st);
// pressure systems; mode 0: pressure (a_P, p0/p1, optional relax),
// 1: correction SIMPLEC (row sums), 2: correction SIMPLE (a_P)
void launch_assemble_pressure(int mode, int relax, const Grid &g, const Phys &ph, const SysView &S,
                              const SysView &U, const SysView &V, const SysView &W, const double *uc,
                              const double *vc, const double *wc, const double *p, cudaStream_t st);
// velocity corrections, face-parallel; kind 0 SIMPLE (a_P), 1 SIMPLEC (row sums)
void launch_correct_velocity(int comp, int simplec, const Grid &g, const Phys &ph, const SysView &A,
                             const double *pc, double *x, double dvmax, cudaStream_t st);
// SIMPLER correction x = x_hat - dp / (a_P d)
void launch_correct_velocity_simpler(int comp, const Grid &g, const Phys &ph, const SysView &A, const double *p,
                                     const double *hat, double *x, double p_0, double p_1, cudaStream_t st);
// revert (iterations()==0 or failure) and optional per-node clamp
// sweep warm start: u, v, w *= ratio; p = p0_new + (p - p0_old) ratio (padded arrays)
void launch_scale_fields(double *u, int nu, double *v, int nv, double *w, int nw, double *p, int np, double ratio,
                         double p0_old, double p0_new, cudaStream_t st);
void launch_velocity_post(const double *temp, double *x, int n, const KState *st_dev, int limit, double dvmax,
                          cudaStream_t st);

// reductions; results land in `out` (device doubles) and are final when the
// stream reaches the end of the launch
struct DiagOut {
    double v_sum, p_out_sum, p_in_sum, cnt_out, cnt_in;     // permeability
    double maxdv, maxdiv, sumdiv2, sumvel;                   // divergence
    double pcmax, pcmin, pcsq;                               // pressure correction
    unsigned int counter[4];
};
void launch_permeability(const Grid &g, const double *u, const double *p, int border, double *part,
                         DiagOut *out, cudaStream_t st);
void launch_divergence(const Grid &g, const Phys &ph, const SysView &P, const double *u, const double *v,
                       const double *w, double *part, DiagOut *out, cudaStream_t st);
void launch_correct_pressure(const SysView &P, const double *pc, double *p, double beta, double *part,
                             DiagOut *out, cudaStream_t st);
void launch_default_pressure(const Grid &g, const SysView &P, double p0, double p1, double *p, cudaStream_t st);
void launch_gather_image(const int *map, long ncells, const double *field, double *img, cudaStream_t st);
void launch_scatter_image(const int *map, long ncells, const double *img, double *field, cudaStream_t st);
void launch_face_average(const Grid &g, const double *u, const double *v, const double *w, double *vavg,
                         cudaStream_t st);

// krylov.cu: batched BiCGSTAB over a set of systems (instantiated for the
// set capacities KMAX and KMAX_MERGED)
template <int CAP>
void launch_krylov_init(const KSetArgT<CAP> &set, cudaStream_t st);
// iterations until every system is done, one needs a restart, or max_iters
// (a merged set takes 1/share of the SMs: `share` merged sets run at once)
template <int CAP>
cudaError_t launch_krylov_loop(const KSetArgT<CAP> &set, GridBar *bar, LoopProf *prof, int max_iters,
                               cudaStream_t st, int share = 1);
template <int CAP>
void launch_krylov_restart(const KSetArgT<CAP> &set, cudaStream_t st);
// blocks of a loop-kernel launch over `units` work units, units_per_chunk
// of them per 1024-row chunk (occ blocks per SM)
int loop_grid(int units, int units_per_chunk, int occ);
// solves running in this process (ns3d_solve calls in flight)
struct ActiveSolve {
    ActiveSolve();
    ~ActiveSolve();
};
int active_solves();
void launch_spmv(const SysView &A, const double *x, double *y, cudaStream_t st);
int device_sm_count();
// kernels launched by this library since it was loaded
int64_t launch_count();
void count_launches(int64_t n);
// zero a loop kernel's grid barrier before a launch (and apply the barrier
// test of ns3d_debug_barrier_timeout while it is set)
cudaError_t reset_grid_bar(GridBar *bar, cudaStream_t st);
void set_barrier_test(unsigned int bias, unsigned long long limit_ns);

}  // namespace ns3d
