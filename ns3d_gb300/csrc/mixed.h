// mixed.h -- data of the mixed-precision (FP32 inner / FP64 outer) solves.
#pragma once

#include "device.cuh"

namespace ns3d {

// work unit of the FP32 loop kernel: MRPL rows per lane, MSUB units per chunk
constexpr int MRPL = 2;
constexpr int MUNIT = LANES * MRPL;
constexpr int MSUB = CH / MUNIT;
static_assert(PART_PER_CHUNK >= 5 * MSUB, "partials of the FP32 loop kernel");

// FP64 defect-correction state of one system
struct DCState {
    double rr, bb, tol, tol2, scale, error, tin, tin_min;
    double theta;    // step length of the current correction (minimal FP64 residual)
    int total_iter, maxit, done, info, zero_rhs;
    int inner_cap;   // FP32 iterations allowed per round
    unsigned int counter, pad2_;
};

// Aggregation multilevel preconditioner of an FP32 inner solve (precision
// mode MIXED_MG, single-system sets): level k+1 aggregates the rows of level
// k by 2x2x2 blocks of their cells; its operator is the Galerkin product
// (sum of the block's couplings; blocks couple through faces only, so it is
// 7-point again, same slot order P,W,E,S,N,B,T).
constexpr int MG_MAX = 6;
struct MGLevel {
    int n, npad;
    const int *nbr;       // [6][npad], -1 none
    float *coef;          // [7][npad]
    float *invdiag;       // [npad]
    const int *agg;       // [rows of level k-1]: the row of this level each belongs to
    const int *mstart;    // [n + 1]: offsets into members
    const int *members;   // rows of level k-1 of each row, ascending
    float *x, *b, *t;     // V-cycle vectors [npad]
};
struct MGSet {
    int nlev;             // coarse levels (0: Jacobi preconditioning)
    int sweeps;           // Jacobi sweeps on the coarsest level
    float omega;          // damping of the Jacobi smoother
    int pad_;
    MGLevel lev[MG_MAX + 1];  // lev[1..nlev]; lev[0] unused (the system itself)
};

struct MSys {
    int n, npad, nchunks, chunk_begin;
    const int *nbr;
    const double *coef64;  // [7][npad]
    const double *b64;     // right-hand side
    double *x64;           // guess in, solution out
    double *r64;           // FP64 residual
    const float *coef32, *invdiag32;
    float *x, *r, *r0, *p, *v, *y, *s, *z, *t;  // FP32 inner vectors (x is the correction)
    float *p2, *v2;  // second buffers of p and v (the loop kernel alternates them)
    double *part;
    KState *st;  // inner BiCGSTAB state (scalars in FP64)
    DCState *dc;
    MGSet mg;
};

// A mixed solve set as a kernel argument (by value; systems in chunk order):
// one solver instance's systems (up to KMAX) or the systems of many
// concurrent solves (up to KMAX_MERGED_M, 24 KB of kernel parameters).
constexpr int KMAX_MERGED_M = 32;
template <int CAP>
struct MSetArgT {
    int nsys, total_chunks;
    MSys sys[CAP];
};
using MSetArg = MSetArgT<KMAX>;
using MSetArgMerged = MSetArgT<KMAX_MERGED_M>;
static_assert(sizeof(MSetArgMerged) <= 32000, "kernel parameter space");

// Galerkin operators of every coarse level of `mg` from the FP32 system
void launch_mg_galerkin(const MSys &sys, cudaStream_t st);
void launch_to_f32(const double *coef, const double *invdiag, int npad, float *coef32, float *invdiag32,
                   cudaStream_t st);
// (the set launchers are instantiated for CAP = KMAX and KMAX_MERGED_M)
template <int CAP>
void launch_dc_resid(const MSetArgT<CAP> &set, int first, cudaStream_t st);
template <int CAP>
void launch_m32_init(const MSetArgT<CAP> &set, cudaStream_t st);
// The FP32 loop variant of a set: fused (three phases per iteration) when
// the set has at most kFusedRows rows and no multilevel system, else the
// five-phase loop.  A merged set runs the variant its members chose alone.
bool m32_fused(long rows, bool mg);
// FP32 inner iterations until every inner solve of the round is done
// (variant: -1 from the set's own rows, 0 five-phase, 1 fused; a merged set
// takes 1/share of the SMs)
template <int CAP>
cudaError_t launch_m32_loop(const MSetArgT<CAP> &set, GridBar *bar, int max_iters, cudaStream_t st,
                            int variant = -1, int share = 1);
// theta = <r, A d> / <A d, A d> for the FP32 correction d (FP64 SpMV), then
// x += theta d
template <int CAP>
void launch_dc_update(const MSetArgT<CAP> &set, cudaStream_t st);

}  // namespace ns3d
