// physics.cu -- assembly, corrections and diagnostics of the NS3D solve.
//
// One thread per row of the system being built (rows are the compacted
// nodes, row -> cell through the `cell` table), so every coefficient is
// written once and coalesced.  The arithmetic of each row follows the
// reference expression by expression (cited per kernel); this file is
// compiled with --fmad=false so nothing is contracted.
#include "device.cuh"
#include "kernels.h"

namespace ns3d {

__device__ __forceinline__ double min0(double F) { return (0.0 < F) ? 0.0 : F; }
__device__ __forceinline__ double max0(double F) { return (F < 0.0) ? 0.0 : F; }

__device__ __forceinline__ void finish_momentum_row(const SysView &A, int r, double D, double aW, double aE, double aS,
                                                    double aN, double aB, double aT) {
    A.c(SP, r) = D;
    A.c(SW, r) = aW;
    A.c(SE, r) = aE;
    A.c(SS, r) = aS;
    A.c(SN, r) = aN;
    A.c(SB, r) = aB;
    A.c(ST, r) = aT;
    const int nW = A.nb(0, r), nE = A.nb(1, r), nS = A.nb(2, r), nN = A.nb(3, r), nB = A.nb(4, r), nT = A.nb(5, r);
    double cf[7] = {D, aW, aE, aS, aN, aB, aT};
    // uA.row(r).sum(): stored entries in ascending column order, plain adds
    A.rowsum[r] = row_ordered(r, nW, nE, nS, nN, nB, nT, [&](double acc, int s, int) { return acc + cf[s]; });
    // DiagonalPreconditioner: 1/a_rr, or 1 for a zero diagonal
    A.invdiag[r] = (D != 0.0) ? 1.0 / D : 1.0;
}

// AssembleMomentum_x, src/NSBase.cxx:886-1057
__global__ void k_mom_x(Grid g, Phys ph, SysView A, const double *__restrict__ uc, const double *__restrict__ vc,
                        const double *__restrict__ wc) {
    const double dx = ph.dx, dy = ph.dy, dz = ph.dz, mu = ph.mu, rho = ph.rho, sf = ph.schemefactor;
    const double idx2 = ph.idx2, idy2 = ph.idy2, idz2 = ph.idz2;
    const double idx = ph.idx, idy = ph.idy, idz = ph.idz;
    const int d0 = g.nx + 1, ny = g.ny, nz = g.nz;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        int i, j, k;
        g.ijk(A.cell[r], i, j, k);
        double D = 0, F, um, vm, wm, Fd;
        double aW = 0, aE = 0, aS = 0, aN = 0, aB = 0, aT = 0;
        const double uC = uc[r];
        const int nE = A.nb(1, r), nW = A.nb(0, r);
        if (i + 1 < d0) {
            if (nE > -1) {
                double uE = uc[nE];
                if (uC > 0 && uE > 0) F = -uC * rho * idx;
                else if (uC < 0 && uE < 0) F = -uE * rho * idx;
                else F = 0;
                if (fabs(F) * dx * dx > 2 * mu * sf) {
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
            if (nW > -1) {
                double uW = uc[nW];
                if (uC < 0 && uW < 0) F = uC * rho * idx;
                else if (uC > 0 && uW > 0) F = uW * rho * idx;
                else F = 0;
                if (fabs(F) * dx * dx > 2 * mu * sf) {
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
            if (A.nb(3, r) > -1) {
                vm = (g.sv(vc, i - 1, j + 1, k) + g.sv(vc, i, j + 1, k)) * 0.5;
                F = -vm * rho * idy;
                if (fabs(vm) * rho * dy > 2 * mu * sf) {
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
            if (A.nb(2, r) > -1) {
                vm = (g.sv(vc, i - 1, j, k) + g.sv(vc, i, j, k)) * 0.5;
                F = vm * rho * idy;
                if (fabs(vm) * dy * rho > 2 * mu * sf) {
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
                if (A.nb(5, r) > -1) {
                    wm = (g.sw(wc, i - 1, j, k + 1) + g.sw(wc, i, j, k + 1)) * 0.5;
                    F = -wm * rho * idz;
                    if (fabs(wm) * rho * dz > 2 * mu * sf) {
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
                if (A.nb(4, r) > -1) {
                    wm = (g.sw(wc, i - 1, j, k) + g.sw(wc, i, j, k)) * 0.5;
                    F = wm * rho * idz;
                    if (fabs(wm) * rho * dz > 2 * mu * sf) {
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
        D /= ph.alpha;
        finish_momentum_row(A, r, D, aW, aE, aS, aN, aB, aT);
    }
}

// AssembleMomentum_y, src/NSBase.cxx:1059-1250
__global__ void k_mom_y(Grid g, Phys ph, SysView A, const double *__restrict__ uc, const double *__restrict__ vc,
                        const double *__restrict__ wc) {
    const double dx = ph.dx, dy = ph.dy, dz = ph.dz, mu = ph.mu, rho = ph.rho, sf = ph.schemefactor;
    const double idx2 = ph.idx2, idy2 = ph.idy2, idz2 = ph.idz2;
    const double idx = ph.idx, idy = ph.idy, idz = ph.idz;
    const int d0 = g.nx, ny = g.ny, nz = g.nz;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        int i, j, k;
        g.ijk(A.cell[r], i, j, k);
        double D = 0, F, um, vm, wm, Fd;
        double aW = 0, aE = 0, aS = 0, aN = 0, aB = 0, aT = 0;
        if (i + 1 < d0) {
            if (A.nb(1, r) > -1) {
                um = (g.su(uc, i + 1, j - 1, k) + g.su(uc, i + 1, j, k)) * 0.5;
                F = -um * rho * idx;
                if (fabs(um) * dx * rho > 2 * mu * sf) {
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
            D += -(0.5 * rho * idx) * (g.su(uc, i + 1, j - 1, k) + g.su(uc, i + 1, j, k));
        }
        if (i - 1 >= 0) {
            if (A.nb(0, r) > -1) {
                um = (g.su(uc, i, j - 1, k) + g.su(uc, i, j, k)) * 0.5;
                F = um * rho * idx;
                if (fabs(um) * dx * rho > 2 * mu * sf) {
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
            D += -mu * idx2 + (0.25 * rho * idx) * (g.su(uc, i, j - 1, k) + g.su(uc, i, j, k));
        }
        const double vC = vc[r];
        const int nN = A.nb(3, r), nS = A.nb(2, r);
        if (j + 1 < ny) {
            if (nN > -1) {
                double vN = vc[nN];
                if (vC > 0 && vN > 0) F = -vC * rho * idy;
                else if (vC < 0 && vN < 0) F = -vN * rho * idy;
                else F = 0;
                if (fabs(F) * dy * dy > 2 * mu * sf) {
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
            if (nS > -1) {
                double vS = vc[nS];
                if (vC < 0 && vS < 0) F = vC * rho * idy;
                else if (vC > 0 && vS > 0) F = vS * rho * idy;
                else F = 0;
                if (fabs(F) * dy * dy > 2 * mu * sf) {
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
                if (A.nb(5, r) > -1) {
                    wm = (g.sw(wc, i, j - 1, k + 1) + g.sw(wc, i, j, k + 1)) * 0.5;
                    F = -wm * rho * idz;
                    if (fabs(wm) * rho * dz > 2 * mu * sf) {
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
                if (A.nb(4, r) > -1) {
                    wm = (g.sw(wc, i, j - 1, k) + g.sw(wc, i, j, k)) * 0.5;
                    F = wm * rho * idz;
                    if (fabs(wm) * rho * dz > 2 * mu * sf) {
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
        D /= ph.alpha;
        finish_momentum_row(A, r, D, aW, aE, aS, aN, aB, aT);
    }
}

// AssembleMomentum_z, src/NSBase.cxx:1252-1442
__global__ void k_mom_z(Grid g, Phys ph, SysView A, const double *__restrict__ uc, const double *__restrict__ vc,
                        const double *__restrict__ wc) {
    const double dx = ph.dx, dy = ph.dy, dz = ph.dz, mu = ph.mu, rho = ph.rho, sf = ph.schemefactor;
    const double idx2 = ph.idx2, idy2 = ph.idy2, idz2 = ph.idz2;
    const double idx = ph.idx, idy = ph.idy, idz = ph.idz;
    const int d0 = g.nx, ny = g.ny, nz = g.nz;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        int i, j, k;
        g.ijk(A.cell[r], i, j, k);
        double D = 0, F, um, vm, wm, Fd;
        double aW = 0, aE = 0, aS = 0, aN = 0, aB = 0, aT = 0;
        if (i + 1 < d0) {
            if (A.nb(1, r) > -1) {
                um = (g.su(uc, i + 1, j, k - 1) + g.su(uc, i + 1, j, k)) * 0.5;
                F = -um * rho * idx;
                if (fabs(um) * dx * rho > 2 * mu * sf) {
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
            D += -(0.5 * rho * idx) * (g.su(uc, i + 1, j, k - 1) + g.su(uc, i + 1, j, k));
        }
        if (i - 1 >= 0) {
            if (A.nb(0, r) > -1) {
                um = (g.su(uc, i, j, k - 1) + g.su(uc, i, j, k)) * 0.5;
                F = um * rho * idx;
                if (fabs(um) * dx * rho > 2 * mu * sf) {
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
            D += -mu * idx2 + (0.25 * rho * idx) * (g.su(uc, i, j, k - 1) + g.su(uc, i, j, k));
        }
        if (j + 1 < ny) {
            if (A.nb(3, r) > -1) {
                vm = (g.sv(vc, i, j + 1, k - 1) + g.sv(vc, i, j + 1, k)) * 0.5;
                F = -vm * rho * idy;
                if (fabs(vm) * rho * dy > 2 * mu * sf) {
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
            if (A.nb(2, r) > -1) {
                vm = (g.sv(vc, i, j, k - 1) + g.sv(vc, i, j, k)) * 0.5;
                F = vm * rho * idy;
                if (fabs(vm) * rho * dy > 2 * mu * sf) {
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
        const double wC = wc[r];
        const int nT = A.nb(5, r), nB = A.nb(4, r);
        if (k + 1 < nz) {
            if (nT > -1) {
                double wT = wc[nT];
                if (wC > 0 && wT > 0) F = -wC * rho * idz;
                else if (wC < 0 && wT < 0) F = -wT * rho * idz;
                else F = 0;
                if (fabs(F) * dz * dz > 2 * mu * sf) {
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
            if (nB > -1) {
                double wB = wc[nB];
                if (wB < 0 && wC < 0) F = wC * rho * idz;
                else if (wB > 0 && wC > 0) F = wB * rho * idz;
                else F = 0;
                if (fabs(F) * dz * dz > 2 * mu * sf) {
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
        D /= ph.alpha;
        finish_momentum_row(A, r, D, aW, aE, aS, aN, aB, aT);
    }
}

// Assemble_RHS_u/v/w, src/NSBase.cxx:1445-1546
template <int COMP>
__global__ void k_mom_rhs(Grid g, Phys ph, SysView A, const double *__restrict__ p, const double *__restrict__ x) {
    const double idx = ph.idx, idy = ph.idy, idz = ph.idz;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        int i, j, k;
        g.ijk(A.cell[r], i, j, k);
        double b;
        if (COMP == 0) {
            if (i == 0) b = (p[g.P(i, j, k)] - ph.p0) * idx;
            else if (i == g.nx) b = (ph.p1 - p[g.P(i - 1, j, k)]) * idx;
            else b = (p[g.P(i, j, k)] - p[g.P(i - 1, j, k)]) * idx;
            b += x[r] * A.c(SP, r) * (1 - ph.alpha);
        } else if (COMP == 1) {
            b = (p[g.P(i, j, k)] - p[g.P(i, j - 1, k)]) * idy + x[r] * A.c(SP, r) * (1 - ph.alpha);
        } else {
            b = (p[g.P(i, j, k)] - p[g.P(i, j, k - 1)]) * idz + x[r] * A.c(SP, r) * (1 - ph.alpha);
        }
        A.rhs[r] = b;
    }
}

// Compute_{u,v,w}_hat, src/NSBase.cxx:1548-1755: subtractions in the order
// E, W, N, S, T, B, then division by the (relaxed) diagonal
__global__ void k_hat(SysView A, Phys ph, const double *__restrict__ xc, const double *__restrict__ xold,
                      double *__restrict__ hat) {
    const int order[6] = {SE, SW, SN, SS, ST, SB};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        double t = 0;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            int s = order[q];
            int c = A.nb(s - 1, r);
            if (c >= 0) t -= A.c(s, r) * xc[c];
        }
        hat[r] = (t) / (A.c(SP, r)) + xold[r] * (1 - ph.alpha);
    }
}

// AssemblePressure (mode 0, src/NSBase.cxx:478-610),
// AssemblePressureCorrectionSIMPLEC (mode 1, :612-732), ...SIMPLE (mode 2, :734-851)
__global__ void k_pressure(int mode, int relax, Grid g, Phys ph, SysView S, const double *__restrict__ au,
                           const double *__restrict__ av, const double *__restrict__ aw, const double *__restrict__ uc,
                           const double *__restrict__ vc, const double *__restrict__ wc, const double *__restrict__ p) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const double dx2 = ph.dx * ph.dx, dy2 = ph.dy * ph.dy, dz2 = ph.dz * ph.dz;
    const double idx = ph.idx, idy = ph.idy, idz = ph.idz;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < S.n; r += gridDim.x * blockDim.x) {
        int i, j, k;
        g.ijk(S.cell[r], i, j, k);
        double D = 0, b = 0;
        double cW = 0, cE = 0, cS = 0, cN = 0, cB = 0, cT = 0;
        int f;
        if (i > 0 && g.P(i - 1, j, k) > -1 && (f = g.U(i, j, k)) > -1) {
            D += 1 / ((au[f]) * dx2);
            cW = -1 / ((au[f]) * dx2);
            b -= uc[f] * idx;
        }
        if (i < nx - 1 && g.P(i + 1, j, k) > -1 && (f = g.U(i + 1, j, k)) > -1) {
            D += 1 / ((au[f]) * dx2);
            cE = -1 / ((au[f]) * dx2);
            b += uc[f] * idx;
        }
        if (j > 0 && g.P(i, j - 1, k) > -1 && (f = g.V(i, j, k)) > -1) {
            D += 1 / ((av[f]) * dy2);
            cS = -1 / ((av[f]) * dy2);
            b -= vc[f] * idy;
        }
        if (j < ny - 1 && g.P(i, j + 1, k) > -1 && (f = g.V(i, j + 1, k)) > -1) {
            D += 1 / ((av[f]) * dy2);
            cN = -1 / ((av[f]) * dy2);
            b += vc[f] * idy;
        }
        if (k > 0 && g.P(i, j, k - 1) > -1 && (f = g.W(i, j, k)) > -1) {
            D += 1 / ((aw[f]) * dz2);
            cB = -1 / ((aw[f]) * dz2);
            b -= wc[f] * idz;
        }
        if (k < nz - 1 && g.P(i, j, k + 1) > -1 && (f = g.W(i, j, k + 1)) > -1) {
            D += 1 / ((aw[f]) * dz2);
            cT = -1 / ((aw[f]) * dz2);
            b += wc[f] * idz;
        }
        if (i == 0 && (f = g.U(i, j, k)) > -1) {
            D += 1 / ((au[f]) * dx2);
            if (mode == 0) b -= uc[f] * idx - ph.p0 / (au[f] * dx2);
            else b -= uc[f] * idx;
        }
        if (i == nx - 1 && (f = g.U(i + 1, j, k)) > -1) {
            D += 1 / ((au[f]) * dx2);
            if (mode == 0) b += uc[f] * idx + ph.p1 / (au[f] * dx2);
            else b += uc[f] * idx;
        }
        if (mode == 0 && relax) {
            D /= ph.beta;
            b += p[r] * D * (1 - ph.beta);
        }
        S.c(SP, r) = D;
        S.c(SW, r) = cW;
        S.c(SE, r) = cE;
        S.c(SS, r) = cS;
        S.c(SN, r) = cN;
        S.c(SB, r) = cB;
        S.c(ST, r) = cT;
        S.rhs[r] = b;
        S.invdiag[r] = (D != 0.0) ? 1.0 / D : 1.0;
    }
}

__device__ __forceinline__ double clampdv(double d, double m) {
    if (d < 0 && fabs(d) > m) d = -m;
    else if (d > 0 && d > m) d = m;
    return d;
}

// CorrectVelocityFieldSIMPLE / ...SIMPLEC (src/NSBase.cxx:2082-2263), one
// thread per face node: each face is corrected by exactly one pressure cell
// (its +side cell, or cell nx-1 for the outlet faces), as in the reference
template <int COMP>
__global__ void k_correct(Grid g, Phys ph, SysView A, const double *__restrict__ den, const double *__restrict__ pc,
                          double *__restrict__ x, double dvmax) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        int i, j, k, q, c;
        g.ijk(A.cell[r], i, j, k);
        double d;
        if (COMP == 0) {
            if (i == g.nx) {  // outlet face, owned by cell nx-1
                c = g.P(i - 1, j, k);
                if (c < 0) continue;
                d = -(pc[c]) / ((den[r]) * ph.dx);
            } else if (i == 0) {  // inlet face
                c = g.P(i, j, k);
                if (c < 0) continue;
                d = (pc[c]) / ((den[r]) * ph.dx);
            } else {
                c = g.P(i, j, k);
                q = g.P(i - 1, j, k);
                if (c < 0 || q < 0) continue;
                d = -(pc[q] - pc[c]) / ((den[r]) * ph.dx);
            }
        } else if (COMP == 1) {
            c = g.P(i, j, k);
            q = (j > 0) ? g.P(i, j - 1, k) : -1;
            if (c < 0 || q < 0) continue;
            d = -(pc[q] - pc[c]) / ((den[r]) * ph.dy);
        } else {
            c = g.P(i, j, k);
            q = (k > 0) ? g.P(i, j, k - 1) : -1;
            if (c < 0 || q < 0) continue;
            d = -(pc[q] - pc[c]) / ((den[r]) * ph.dz);
        }
        x[r] = x[r] + clampdv(d, dvmax);
    }
}

// CorrectVelocityFieldSIMPLER, src/NSBase.cxx:2265-2335 (face-parallel)
template <int COMP>
__global__ void k_correct_simpler(Grid g, Phys ph, SysView A, const double *__restrict__ p,
                                  const double *__restrict__ hat, double *__restrict__ x, double p_0, double p_1) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n; r += gridDim.x * blockDim.x) {
        int i, j, k, q, c;
        g.ijk(A.cell[r], i, j, k);
        const double a = A.c(SP, r);
        if (COMP == 0) {
            if (i == g.nx) {
                c = g.P(i - 1, j, k);
                if (c < 0) continue;
                x[r] = hat[r] - (p[c] - p_1) / (a * ph.dx);
            } else if (i == 0) {
                c = g.P(i, j, k);
                if (c < 0) continue;
                x[r] = hat[r] - (p_0 - p[c]) / (a * ph.dx);
            } else {
                c = g.P(i, j, k);
                q = g.P(i - 1, j, k);
                if (c < 0 || q < 0) continue;
                x[r] = hat[r] - (p[q] - p[c]) / (a * ph.dx);
            }
        } else if (COMP == 1) {
            c = g.P(i, j, k);
            q = (j > 0) ? g.P(i, j - 1, k) : -1;
            if (c < 0 || q < 0) continue;
            x[r] = hat[r] - (p[q] - p[c]) / (a * ph.dy);
        } else {
            c = g.P(i, j, k);
            q = (k > 0) ? g.P(i, j, k - 1) : -1;
            if (c < 0 || q < 0) continue;
            x[r] = hat[r] - (p[q] - p[c]) / (a * ph.dz);
        }
    }
}

// ComputeVelocityField tail, src/NSBase.cxx:1800-1818: keep the previous
// field when the solve took 0 iterations or failed, then clamp the update
__global__ void k_velocity_post(const double *__restrict__ temp, double *__restrict__ x, int n,
                                const KState *__restrict__ st, int limit, double dvmax) {
    const bool revert = (st->iter == 0) || (st->info != 0);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double t = temp[r];
        double v = revert ? t : x[r];
        if (limit) {
            double d = v - t;
            if (fabs(d) > dvmax) {
                if (d > 0) v = t + dvmax;
                else if (d < 0) v = t - dvmax;
            }
        }
        x[r] = v;
    }
}

// ---- reductions with last-block completion ---------------------------------
// Each block reduces whole 1024-row chunks; the block that completes the last
// chunk combines the chunk partials in fixed order and publishes the result.
__device__ __forceinline__ bool last_block_arrive(unsigned int *counter, unsigned int total, bool *sh_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        *sh_flag = (prev == total - 1);
    }
    __syncthreads();
    bool last = *sh_flag;
    if (last) __threadfence();
    return last;
}

// ComputePermeability, src/NSBase.cxx:1886-1956: sums over the outlet u plane
// (and, with a border, the inlet/outlet p planes), positions q = j*nz + k
__global__ void k_permeability(Grid g, const double *__restrict__ u, const double *__restrict__ p, int border,
                               double *__restrict__ part, DiagOut *out) {
    __shared__ double sm[LANES];
    __shared__ bool last;
    const long plane = (long)g.ny * g.nz;
    const int nch = (int)((plane + CH - 1) / CH);
    const int iu = (border <= 0) ? g.nx : g.nx + 1 - border;
    const int io = g.nx - border, ii = border - 1;
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        double a = 0, so = 0, si = 0, co = 0, ci = 0;
        for (int m = 0; m < RPL; ++m) {
            long q = (long)c * CH + threadIdx.x + LANES * m;
            if (q >= plane) break;
            int r = g.umap[(long)iu * plane + q];
            if (r > -1) a = a + u[r];
            if (border > 0) {
                int ro = g.pmap[(long)io * plane + q];
                if (ro > -1) { so = so + p[ro]; co = co + 1.0; }
                int ri = g.pmap[(long)ii * plane + q];
                if (ri > -1) { si = si + p[ri]; ci = ci + 1.0; }
            }
        }
        double ta = block_tree_sum(a, sm);
        double tso = block_tree_sum(so, sm);
        double tsi = block_tree_sum(si, sm);
        double tco = block_tree_sum(co, sm);
        double tci = block_tree_sum(ci, sm);
        if (threadIdx.x == 0) {
            part[(size_t)c * 5 + 0] = ta;
            part[(size_t)c * 5 + 1] = tso;
            part[(size_t)c * 5 + 2] = tsi;
            part[(size_t)c * 5 + 3] = tco;
            part[(size_t)c * 5 + 4] = tci;
        }
        if (last_block_arrive(&out->counter[0], (unsigned)nch, &last)) {
            double fa = final_partials_sum(part + 0, nch, 5, sm);
            double fo = final_partials_sum(part + 1, nch, 5, sm);
            double fi = final_partials_sum(part + 2, nch, 5, sm);
            double fco = final_partials_sum(part + 3, nch, 5, sm);
            double fci = final_partials_sum(part + 4, nch, 5, sm);
            if (threadIdx.x == 0) {
                out->v_sum = fa;
                out->p_out_sum = fo;
                out->p_in_sum = fi;
                out->cnt_out = fco;
                out->cnt_in = fci;
                out->counter[0] = 0;
            }
        }
    }
}

// ComputeDiv, src/NSBase.cxx:1958-2080
__global__ void k_divergence(Grid g, Phys ph, SysView P, const double *__restrict__ u, const double *__restrict__ v,
                             const double *__restrict__ w, double *__restrict__ part, DiagOut *out) {
    __shared__ double sm[LANES];
    __shared__ bool last;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const double idx = ph.idx, idy = ph.idy, idz = ph.idz;
    for (int c = blockIdx.x; c < P.nchunks; c += gridDim.x) {
        double s2 = 0, sv = 0, mdv = 0, mdiv = 0;
        for (int m = 0; m < RPL; ++m) {
            int r = c * CH + threadIdx.x + LANES * m;
            if (r >= P.n) break;
            int i, j, k, f;
            g.ijk(P.cell[r], i, j, k);
            double div = 0, uu = 0, vv = 0, ww = 0, DV = 0;
            if (i > 0 && g.P(i - 1, j, k) > -1 && (f = g.U(i, j, k)) > -1) {
                div += -u[f] * idx; DV += -u[f]; uu += u[f] * 0.5;
            }
            if (i < nx - 1 && g.P(i + 1, j, k) > -1 && (f = g.U(i + 1, j, k)) > -1) {
                div += u[f] * idx; DV += u[f]; uu += u[f] * 0.5;
            }
            if (j > 0 && g.P(i, j - 1, k) > -1 && (f = g.V(i, j, k)) > -1) {
                div += -v[f] * idy; DV += -v[f]; vv += v[f] * 0.5;
            }
            if (j < ny - 1 && g.P(i, j + 1, k) > -1 && (f = g.V(i, j + 1, k)) > -1) {
                div += v[f] * idy; DV += v[f]; vv += v[f] * 0.5;
            }
            if (k > 0 && g.P(i, j, k - 1) > -1 && (f = g.W(i, j, k)) > -1) {
                div += -w[f] * idz; DV += -w[f]; ww += w[f] * 0.5;
            }
            if (k < nz - 1 && g.P(i, j, k + 1) > -1 && (f = g.W(i, j, k + 1)) > -1) {
                div += w[f] * idz; DV += w[f]; ww += w[f] * 0.5;
            }
            if (i == 0 && (f = g.U(i, j, k)) > -1) {
                div += -u[f] * idx; DV += -u[f]; uu += u[f] * 0.5;
            }
            if (i == nx - 1 && (f = g.U(i + 1, j, k)) > -1) {
                div += u[f] * idx; DV += u[f]; uu += u[f] * 0.5;
            }
            DV = fabs(DV);
            div = fabs(div);
            mdv = dmaxv(mdv, DV);
            mdiv = dmaxv(mdiv, div);
            s2 = __fma_rn(div, div, s2);
            sv = sv + sqrt(uu * uu + vv * vv + ww * ww);
        }
        double t2 = block_tree_sum(s2, sm);
        double tv = block_tree_sum(sv, sm);
        double tm1 = block_tree_max(mdv, sm);
        double tm2 = block_tree_max(mdiv, sm);
        if (threadIdx.x == 0) {
            part[(size_t)c * 4 + 0] = t2;
            part[(size_t)c * 4 + 1] = tv;
            part[(size_t)c * 4 + 2] = tm1;
            part[(size_t)c * 4 + 3] = tm2;
        }
        if (last_block_arrive(&out->counter[1], (unsigned)P.nchunks, &last)) {
            double f2 = final_partials_sum(part + 0, P.nchunks, 4, sm);
            double fv = final_partials_sum(part + 1, P.nchunks, 4, sm);
            double m1 = 0, m2 = 0;
            for (int q = threadIdx.x; q < P.nchunks; q += LANES) {
                m1 = dmaxv(m1, __ldcg(part + (size_t)q * 4 + 2));
                m2 = dmaxv(m2, __ldcg(part + (size_t)q * 4 + 3));
            }
            m1 = block_tree_max(m1, sm);
            m2 = block_tree_max(m2, sm);
            if (threadIdx.x == 0) {
                out->sumdiv2 = f2;
                out->sumvel = fv;
                out->maxdv = m1;
                out->maxdiv = m2;
                out->counter[1] = 0;
            }
        }
    }
}

// CorrectPressureField, src/NSBase.cxx:2367-2380: max, min, |pc|^2, p += beta pc
__global__ void k_correct_pressure(SysView P, const double *__restrict__ pc, double *__restrict__ p, double beta,
                                   double *__restrict__ part, DiagOut *out) {
    __shared__ double sm[LANES];
    __shared__ bool last;
    for (int c = blockIdx.x; c < P.nchunks; c += gridDim.x) {
        double mx = -HUGE_VAL, mn = HUGE_VAL, sq = 0;
        for (int m = 0; m < RPL; ++m) {
            int r = c * CH + threadIdx.x + LANES * m;
            if (r >= P.n) break;
            double x = pc[r];
            mx = (x > mx) ? x : mx;
            mn = (x < mn) ? x : mn;
            sq = __fma_rn(x, x, sq);
            p[r] = p[r] + beta * x;
        }
        double tmx = block_tree_max(mx, sm);
        double tmn = block_tree_min(mn, sm);
        double tsq = block_tree_sum(sq, sm);
        if (threadIdx.x == 0) {
            part[(size_t)c * 3 + 0] = tmx;
            part[(size_t)c * 3 + 1] = tmn;
            part[(size_t)c * 3 + 2] = tsq;
        }
        if (last_block_arrive(&out->counter[2], (unsigned)P.nchunks, &last)) {
            double fsq = final_partials_sum(part + 2, P.nchunks, 3, sm);
            double a = -HUGE_VAL, b = HUGE_VAL;
            for (int q = threadIdx.x; q < P.nchunks; q += LANES) {
                a = dmaxv(a, __ldcg(part + (size_t)q * 3 + 0));
                b = dminv(b, __ldcg(part + (size_t)q * 3 + 1));
            }
            a = block_tree_max(a, sm);
            b = block_tree_min(b, sm);
            if (threadIdx.x == 0) {
                out->pcmax = a;
                out->pcmin = b;
                out->pcsq = fsq;
                out->counter[2] = 0;
            }
        }
    }
}

// Initpvector default profile, src/NSBase.cxx:2671-2681
__global__ void k_default_pressure(Grid g, SysView P, double p0, double p1, double *__restrict__ p) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < P.n; r += gridDim.x * blockDim.x) {
        int i, j, k;
        g.ijk(P.cell[r], i, j, k);
        p[r] = (p1 - p0) * ((double)i + 1.0) / ((double)g.nx) + p0;
    }
}

__global__ void k_gather_image(const int *__restrict__ map, long ncells, const double *__restrict__ f,
                               double *__restrict__ img) {
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += (long)gridDim.x * blockDim.x) {
        int r = map[c];
        img[c] = r > -1 ? f[r] : 0.0;
    }
}
__global__ void k_scatter_image(const int *__restrict__ map, long ncells, const double *__restrict__ img,
                                double *__restrict__ f) {
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += (long)gridDim.x * blockDim.x) {
        int r = map[c];
        if (r != -1) f[r] = img[c];
    }
}

// FieldsToImage face averages, src/NSBase.cxx:425-466
__global__ void k_face_average(Grid g, const double *__restrict__ u, const double *__restrict__ v,
                               const double *__restrict__ w, double *__restrict__ out) {
    const long N = (long)g.nx * g.ny * g.nz;
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += (long)gridDim.x * blockDim.x) {
        int i, j, k;
        g.ijk(c, i, j, k);
        double au = 0, av = 0, aw = 0;
        int a = g.U(i + 1, j, k), b = g.U(i, j, k);
        if (a > -1 && b > -1) au = (u[a] + u[b]) * 0.50;
        else if (a > -1) au = (u[a]) * 0.50;
        else if (b > -1) au = (u[b]) * 0.50;
        b = g.V(i, j, k);
        if (j < g.ny - 1) {
            a = g.V(i, j + 1, k);
            if (a > -1 && b > -1) av = (v[a] + v[b]) * 0.50;
            else if (a > -1) av = (v[a]) * 0.50;
            else if (b > -1) av = (v[b]) * 0.50;
        } else if (b > -1) av = (v[b]) * 0.50;
        b = g.W(i, j, k);
        if (k < g.nz - 1) {
            a = g.W(i, j, k + 1);
            if (a > -1 && b > -1) aw = (w[a] + w[b]) * 0.50;
            else if (a > -1) aw = (w[a]) * 0.50;
            else if (b > -1) aw = (w[b]) * 0.50;
        } else if (b > -1) aw = (w[b]) * 0.50;
        out[3 * c + 0] = au;
        out[3 * c + 1] = av;
        out[3 * c + 2] = aw;
    }
}

// warm start of a pressure-drop sweep: u, v, w *= ratio; p = p0' + (p - p0) ratio
__global__ void k_scale_fields(double *u, int nu, double *v, int nv, double *w, int nw, double *p, int np,
                               double ratio, double p0_old, double p0_new) {
    const long total = (long)nu + nv + nw + np;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        if (i < nu) u[i] = u[i] * ratio;
        else if (i < (long)nu + nv) v[i - nu] = v[i - nu] * ratio;
        else if (i < (long)nu + nv + nw) w[i - nu - nv] = w[i - nu - nv] * ratio;
        else {
            const long k = i - nu - nv - nw;
            p[k] = p0_new + (p[k] - p0_old) * ratio;
        }
    }
}

// ---- launchers ---------------------------------------------------------------
static inline int rows_grid(long n) { return (int)std::max<long>(1, std::min<long>((n + 255) / 256, 152L * 16)); }
static inline int chunk_grid(int nch) { return std::max(1, std::min(nch, 152 * 8)); }

void launch_assemble_momentum(int comp, const Grid &g, const Phys &ph, const SysView &A, const double *uc,
                              const double *vc, const double *wc, cudaStream_t st) {
    if (A.n <= 0) return;
    if (comp == 0) { count_launches(1); k_mom_x<<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, uc, vc, wc); }
    else if (comp == 1) { count_launches(1); k_mom_y<<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, uc, vc, wc); }
    else { count_launches(1); k_mom_z<<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, uc, vc, wc); }
}

void launch_momentum_rhs(int comp, const Grid &g, const Phys &ph, const SysView &A, const double *p,
                         const double *x, cudaStream_t st) {
    if (A.n <= 0) return;
    if (comp == 0) { count_launches(1); k_mom_rhs<0><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, p, x); }
    else if (comp == 1) { count_launches(1); k_mom_rhs<1><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, p, x); }
    else { count_launches(1); k_mom_rhs<2><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, p, x); }
}

void launch_hat(const SysView &A, const Phys &ph, const double *xc, const double *xold, double *hat,
                cudaStream_t st) {
    if (A.n <= 0) return;
    count_launches(1); k_hat<<<rows_grid(A.n), 256, 0, st>>>(A, ph, xc, xold, hat);
}

void launch_assemble_pressure(int mode, int relax, const Grid &g, const Phys &ph, const SysView &S,
                              const SysView &U, const SysView &V, const SysView &W, const double *uc,
                              const double *vc, const double *wc, const double *p, cudaStream_t st) {
    if (S.n <= 0) return;
    const double *au = (mode == 1) ? U.rowsum : U.coef;  // slot P is the first slot
    const double *av = (mode == 1) ? V.rowsum : V.coef;
    const double *aw = (mode == 1) ? W.rowsum : W.coef;
    count_launches(1); k_pressure<<<rows_grid(S.n), 256, 0, st>>>(mode, relax, g, ph, S, au, av, aw, uc, vc, wc, p);
}

void launch_correct_velocity(int comp, int simplec, const Grid &g, const Phys &ph, const SysView &A,
                             const double *pc, double *x, double dvmax, cudaStream_t st) {
    if (A.n <= 0) return;
    const double *den = simplec ? A.rowsum : A.coef;
    if (comp == 0) { count_launches(1); k_correct<0><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, den, pc, x, dvmax); }
    else if (comp == 1) { count_launches(1); k_correct<1><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, den, pc, x, dvmax); }
    else { count_launches(1); k_correct<2><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, den, pc, x, dvmax); }
}

void launch_correct_velocity_simpler(int comp, const Grid &g, const Phys &ph, const SysView &A, const double *p,
                                     const double *hat, double *x, double p_0, double p_1, cudaStream_t st) {
    if (A.n <= 0) return;
    if (comp == 0) { count_launches(1); k_correct_simpler<0><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, p, hat, x, p_0, p_1); }
    else if (comp == 1) { count_launches(1); k_correct_simpler<1><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, p, hat, x, p_0, p_1); }
    else { count_launches(1); k_correct_simpler<2><<<rows_grid(A.n), 256, 0, st>>>(g, ph, A, p, hat, x, p_0, p_1); }
}

void launch_scale_fields(double *u, int nu, double *v, int nv, double *w, int nw, double *p, int np, double ratio,
                         double p0_old, double p0_new, cudaStream_t st) {
    count_launches(1);
    k_scale_fields<<<152 * 8, 256, 0, st>>>(u, nu, v, nv, w, nw, p, np, ratio, p0_old, p0_new);
}

void launch_velocity_post(const double *temp, double *x, int n, const KState *st_dev, int limit, double dvmax,
                          cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1); k_velocity_post<<<rows_grid(n), 256, 0, st>>>(temp, x, n, st_dev, limit, dvmax);
}

void launch_permeability(const Grid &g, const double *u, const double *p, int border, double *part, DiagOut *out,
                         cudaStream_t st) {
    long plane = (long)g.ny * g.nz;
    int nch = (int)((plane + CH - 1) / CH);
    count_launches(1); k_permeability<<<chunk_grid(nch), LANES, 0, st>>>(g, u, p, border, part, out);
}

void launch_divergence(const Grid &g, const Phys &ph, const SysView &P, const double *u, const double *v,
                       const double *w, double *part, DiagOut *out, cudaStream_t st) {
    if (P.n <= 0) {
        cudaMemsetAsync(&out->maxdv, 0, 4 * sizeof(double), st);
        return;
    }
    count_launches(1); k_divergence<<<chunk_grid(P.nchunks), LANES, 0, st>>>(g, ph, P, u, v, w, part, out);
}

void launch_correct_pressure(const SysView &P, const double *pc, double *p, double beta, double *part,
                             DiagOut *out, cudaStream_t st) {
    if (P.n <= 0) return;
    count_launches(1); k_correct_pressure<<<chunk_grid(P.nchunks), LANES, 0, st>>>(P, pc, p, beta, part, out);
}

void launch_default_pressure(const Grid &g, const SysView &P, double p0, double p1, double *p, cudaStream_t st) {
    if (P.n <= 0) return;
    count_launches(1); k_default_pressure<<<rows_grid(P.n), 256, 0, st>>>(g, P, p0, p1, p);
}

void launch_gather_image(const int *map, long ncells, const double *field, double *img, cudaStream_t st) {
    count_launches(1); k_gather_image<<<rows_grid(ncells), 256, 0, st>>>(map, ncells, field, img);
}
void launch_scatter_image(const int *map, long ncells, const double *img, double *field, cudaStream_t st) {
    count_launches(1); k_scatter_image<<<rows_grid(ncells), 256, 0, st>>>(map, ncells, img, field);
}
void launch_face_average(const Grid &g, const double *u, const double *v, const double *w, double *vavg,
                         cudaStream_t st) {
    long N = (long)g.nx * g.ny * g.nz;
    count_launches(1); k_face_average<<<rows_grid(N), 256, 0, st>>>(g, u, v, w, vavg);
}

}  // namespace ns3d
