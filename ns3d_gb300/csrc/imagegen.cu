// imagegen.cu -- seeded synthetic porous images rasterised on the device.
//
// The reference reads its geometry from .vti files; the serving and batch
// workloads need many seeded images (sphere and fibre packs of given
// porosity).  The primitives are drawn on the host from a seeded splitmix64
// stream (no transcendental functions, so the same seed gives the same
// primitives on every host), the device stamps them:
//   kind 0: overlapping balls of integer radius R, integer centres uniform in
//           the box;
//   kind 1: isotropic straight fibres: a point uniform in the box and a
//           direction uniform on the sphere (rejection sampling in the cube);
//           the fibre is the union of balls of radius R centred at
//           rint(p + t d), t = -L, -L+1, ..., L-1 (L = box diagonal), those
//           within R of the box.
// Primitives are added in order until the solid fraction reaches
// 1 - porosity: every voxel records the first primitive that covers it
// (atomicMin, independent of the order of the writes), a histogram of those
// indices gives the solid count after k primitives, and the smallest k that
// reaches the target decides the image.
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/ns3d_capi.h"
#include "runtime.h"

namespace ns3d {
namespace {

struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
};

// primitive i: 6 doubles (sphere: centre, 0 0 0; fibre: point, unit direction)
void draw_primitives(int kind, const int n[3], uint64_t seed, int count, std::vector<double> &out) {
    SplitMix rng{seed};
    out.resize((size_t)6 * count);
    for (int i = 0; i < count; ++i) {
        double *q = &out[(size_t)6 * i];
        if (kind == 0) {
            for (int a = 0; a < 3; ++a) q[a] = (double)(rng.next() % (uint64_t)n[a]);
            q[3] = q[4] = q[5] = 0.0;
        } else {
            for (int a = 0; a < 3; ++a) q[a] = rng.uniform() * n[a];
            double d[3], r2;
            do {
                for (int a = 0; a < 3; ++a) d[a] = 2.0 * rng.uniform() - 1.0;
                r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            } while (!(r2 > 1e-12 && r2 <= 1.0));
            const double r = std::sqrt(r2);
            for (int a = 0; a < 3; ++a) q[3 + a] = d[a] / r;
        }
    }
}

struct GenGeom {
    int nx, ny, nz, R, nball, nsteps;
    double L;
};

__device__ __forceinline__ void stamp_one(const GenGeom &g, int *first, int prim, long cx, long cy, long cz,
                                          int b) {
    // b-th offset of the (2R+1)^3 cube; kept when inside the ball
    const int w = 2 * g.R + 1;
    const int ox = b / (w * w) - g.R, oy = (b / w) % w - g.R, oz = b % w - g.R;
    if (ox * ox + oy * oy + oz * oz > g.R * g.R) return;
    const long x = cx + ox, y = cy + oy, z = cz + oz;
    if (x < 0 || y < 0 || z < 0 || x >= g.nx || y >= g.ny || z >= g.nz) return;
    atomicMin(first + ((size_t)z * g.ny + y) * g.nx + x, prim);
}

__global__ void k_stamp_balls(GenGeom g, const double *__restrict__ prims, int nprims, int *first) {
    const long total = (long)nprims * g.nball;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int p = (int)(t / g.nball), b = (int)(t % g.nball);
        const double *q = prims + (size_t)6 * p;
        stamp_one(g, first, p, (long)q[0], (long)q[1], (long)q[2], b);
    }
}

__global__ void k_stamp_fibres(GenGeom g, const double *__restrict__ prims, int nprims, int *first) {
    const long per = (long)g.nsteps * g.nball;
    const long total = (long)nprims * per;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int p = (int)(t / per);
        const long rem = t % per;
        const int s = (int)(rem / g.nball), b = (int)(rem % g.nball);
        const double *q = prims + (size_t)6 * p;
        const double tt = -g.L + (double)s;
        const long cx = (long)rint(q[0] + tt * q[3]);
        const long cy = (long)rint(q[1] + tt * q[4]);
        const long cz = (long)rint(q[2] + tt * q[5]);
        if (cx < -g.R || cy < -g.R || cz < -g.R || cx >= g.nx + g.R || cy >= g.ny + g.R || cz >= g.nz + g.R) continue;
        stamp_one(g, first, p, cx, cy, cz, b);
    }
}

__global__ void k_first_histogram(const int *__restrict__ first, long nvox, int nprims, unsigned int *hist) {
    for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nvox; v += (long)gridDim.x * blockDim.x) {
        const int f = first[v];
        if (f < nprims) atomicAdd(hist + f, 1u);
    }
}

__global__ void k_threshold(const int *__restrict__ first, long nvox, int k, uint8_t *img) {
    for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nvox; v += (long)gridDim.x * blockDim.x)
        img[v] = first[v] < k ? 1 : 0;
}

}  // namespace
}  // namespace ns3d

using namespace ns3d;

extern "C" NS3D_API int ns3d_generate_image(int32_t kind, int32_t nx, int32_t ny, int32_t nz, int32_t radius,
                                            double porosity, uint64_t seed, uint8_t *raw, double *achieved,
                                            double *prims_out, int32_t max_prims, int32_t *nprims_out) {
    if ((kind != 0 && kind != 1) || nx <= 0 || ny <= 0 || nz <= 0 || radius < 0 || radius > 64 ||
        !(porosity >= 0.0 && porosity <= 1.0))
        return report_error(NS3D_ERR_ARG, "ns3d_generate_image: bad kind, size, radius or porosity");
    const long nvox = (long)nx * ny * nz;
    if (nvox > 0x7fffffffL) return report_error(NS3D_ERR_ARG, "ns3d_generate_image: image too large");
    try {
        cudaStream_t st;
        NS3D_CUDA_CHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        OwnedStream owned;
        owned.s = st;
        const int n[3] = {nx, ny, nz};
        GenGeom g;
        g.nx = nx;
        g.ny = ny;
        g.nz = nz;
        g.R = radius;
        g.nball = (2 * radius + 1) * (2 * radius + 1) * (2 * radius + 1);
        g.L = std::sqrt((double)nx * nx + (double)ny * ny + (double)nz * nz);
        g.nsteps = (int)std::ceil(2.0 * g.L);  // t = -L, -L+1, ... < L
        const double target = 1.0 - porosity;
        DBuf<int> first;
        first.alloc(nvox, st);
        DBuf<uint8_t> img;
        img.alloc(nvox, st);
        std::vector<double> prims;
        std::vector<unsigned int> hist;
        int count = 16, k = -1;
        long solid = 0;
        while (true) {
            // the primitive stream is a prefix of every longer one
            draw_primitives(kind, n, seed, count, prims);
            DBuf<double> dprims;
            dprims.alloc(prims.size(), st);
            DBuf<unsigned int> dhist;
            dhist.alloc_zero(count, st);
            NS3D_CUDA_CHECK(cudaMemcpyAsync(dprims.p, prims.data(), prims.size() * 8, cudaMemcpyHostToDevice, st));
            NS3D_CUDA_CHECK(cudaMemsetAsync(first.p, 0x7f, nvox * sizeof(int), st));  // INT_MAX-like
            count_launches(2);
            if (kind == 0) k_stamp_balls<<<1216, 256, 0, st>>>(g, dprims.p, count, first.p);
            else k_stamp_fibres<<<1216, 256, 0, st>>>(g, dprims.p, count, first.p);
            NS3D_CUDA_CHECK(cudaGetLastError());
            k_first_histogram<<<1216, 256, 0, st>>>(first.p, nvox, count, dhist.p);
            NS3D_CUDA_CHECK(cudaGetLastError());
            hist.resize(count);
            NS3D_CUDA_CHECK(cudaMemcpyAsync(hist.data(), dhist.p, count * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                            st));
            NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
            solid = 0;
            // add primitives while the solid fraction is below the target
            k = 0;
            while (k < count && (double)solid / (double)nvox < target) solid += hist[k++];
            if ((double)solid / (double)nvox >= target || target <= 0.0) break;
            if (count >= (1 << 22)) throw ApiError(NS3D_ERR_ARG, "porosity target not reachable");
            count *= 2;
        }
        count_launches(1);
        k_threshold<<<1216, 256, 0, st>>>(first.p, nvox, k, img.p);
        NS3D_CUDA_CHECK(cudaGetLastError());
        if (raw) NS3D_CUDA_CHECK(cudaMemcpyAsync(raw, img.p, nvox, cudaMemcpyDeviceToHost, st));
        NS3D_CUDA_CHECK(cudaStreamSynchronize(st));
        if (achieved) *achieved = 1.0 - (double)solid / (double)nvox;
        if (nprims_out) *nprims_out = k;
        if (prims_out) std::memcpy(prims_out, prims.data(), sizeof(double) * 6 * (size_t)std::min(k, max_prims));
        return NS3D_OK;
    } catch (const ApiError &e) {
        return report_error(e.code, e.what());
    } catch (const std::exception &e) {
        return report_error(NS3D_ERR_CUDA, e.what());
    }
}
