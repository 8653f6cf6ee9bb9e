// main.cpp -- the NS3D program on the GB300 library: same argv contract as
// the reference (src/navierstokes3D.cxx:480-545): `NS3D <file.ini>`,
// `NS3D -h`; exit status 1 on an input error.
#include <cstdio>
#include <cstring>

#include "../../include/ns3d_capi.h"

static void usage() {
    printf("Usage: NS3D <input-file>   (or 'NS3D -h' for this help)\n");
    printf("\nInput file format: one 'key = value' per line.\n");
    printf("Keys are case-insensitive, blank lines and lines starting\n");
    printf("with '#' are ignored, and an inline '# ...' comment is\n");
    printf("allowed after a value. Unknown keys are reported as a warning.\n");
    printf("\nAccepted keys:\n");
    printf("  input          image file (binary 3D image, .vti or .vtk)   [required]\n");
    printf("  pressurefield  initial pressure field file ('none' to skip)\n");
    printf("  vxfield        initial x-velocity field file ('none' to skip)\n");
    printf("  vyfield        initial y-velocity field file ('none' to skip)\n");
    printf("  vzfield        initial z-velocity field file ('none' to skip)\n");
    printf("  dx, dy, dz     grid spacing (m); dy/dz < 0 means 'same as dx'\n");
    printf("  mu             dynamic viscosity (Pa.s)\n");
    printf("  rho            density (kg/m^3)\n");
    printf("  p0             inlet pressure (Pa)\n");
    printf("  gradp          imposed pressure gradient (Pa/m)\n");
    printf("  alpha          velocity relaxation parameter\n");
    printf("  beta           pressure relaxation parameter\n");
    printf("  vsolvertol     velocity solver tolerance\n");
    printf("  psolvertol     pressure solver tolerance\n");
    printf("  pcsolvertol    pressure correction solver tolerance\n");
    printf("  simpletol      outer-loop convergence threshold (relative RMR)\n");
    printf("  deltaRMR       oscillation detection threshold\n");
    printf("  maxitsolver    max iterations of the linear solvers\n");
    printf("  maxitSIMPLE    max outer iterations\n");
    printf("  N1             inner pressure iterations (SIMPLER/SIMPLERR/IDEAL)\n");
    printf("  N2             inner final iterations (IDEAL)\n");
    printf("  save_step      save a field snapshot every N outer iterations\n");
    printf("  porevalue      voxel value of the fluid (0 or 1)\n");
    printf("  direction      pressure gradient direction: 1=x, 2=y, 3=z\n");
    printf("  border         solid border thickness added along x (voxels)\n");
    printf("  method         algorithm: SIMPLEC, SIMPLER, SIMPLERR or IDEAL\n");
    printf("  precision      inner-solve arithmetic: FP64 (default), MIXED, or MIXED_MG\n");
    printf("                 (MIXED with a multilevel preconditioner in the pressure solves)\n");
}

int main(int argc, char **argv) {
    if (argc < 2) {
        usage();
        return 1;
    }
    if (!strcmp(argv[1], "-h") || !strcmp(argv[1], "--help")) {
        usage();
        return 0;
    }
    int rc = ns3d_run_ini(argv[1], nullptr, nullptr);
    return rc == NS3D_OK ? 0 : 1;
}
