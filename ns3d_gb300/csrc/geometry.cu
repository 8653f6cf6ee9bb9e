// geometry.cu -- binarize/rotate/pad the voxel image and build the index maps
// on the device.
//
// The reference numbers the nodes with one sequential scan in (i, j, k)
// order, k fastest (NavierStokesBase::InitIndexArrays,
// src/NSBase.cxx:2495-2573).  Here the same numbering is produced by a
// three-pass parallel scan: per-cell counts of the four kinds of nodes, an
// exclusive scan of the per-block totals, and a scatter that rescans inside
// each block.  A cell contributes at most one p node, one v node, one w node
// and up to two u nodes (its west face, and for i = nx-1 the outlet face
// numbered right after it), which reproduces the u numbering key
// (min(i,nx-1), j, k, i) of the reference bit for bit.
#include "device.cuh"
#include "kernels.h"

namespace ns3d {

constexpr int GEO_THREADS = 256;
constexpr int GEO_CELLS = GEO_THREADS * 4;  // cells per block

// raw (VTK order, x fastest) -> binary image in the solver frame, C order.
// readvtkfile_uint8 src/vtkio.cxx:96-150, Rotation src/NSBase.cxx:2451-2492,
// AddBorder src/NSBase.cxx:2425-2448 (the border is filled with 0 = fluid).
__global__ void k_build_image(const uint8_t *__restrict__ raw, int rnx, int rny, int rnz, int dir, int border,
                              uint8_t pv, uint8_t *__restrict__ img, int nx, int ny, int nz) {
    const long N = (long)nx * ny * nz;
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += (long)gridDim.x * blockDim.x) {
        int K = (int)(c % nz);
        long t = c / nz;
        int J = (int)(t % ny);
        int I = (int)(t / ny) - border;
        int nx0 = nx - 2 * border;
        uint8_t out = 0;
        if (I >= 0 && I < nx0) {
            int i, j, k;
            if (dir == 2) {  // temp(j, nx-1-i, k) = img(i, j, k)
                i = rnx - 1 - J; j = I; k = K;
            } else if (dir == 3) {  // temp(k, j, i) = img(i, j, k)
                i = K; j = J; k = I;
            } else {
                i = I; j = J; k = K;
            }
            uint8_t r = raw[((long)k * rny + j) * rnx + i];
            out = (r == pv) ? 0 : 1;
        }
        img[c] = out;
    }
}

struct CellCounts {
    int p, u, v, w;
};

__device__ __forceinline__ CellCounts cell_counts(const uint8_t *img, int nx, int ny, int nz, long c, int &i, int &j,
                                                  int &k, int &u_west, int &u_out) {
    CellCounts r = {0, 0, 0, 0};
    u_west = 0;
    u_out = 0;
    k = (int)(c % nz);
    long t = c / nz;
    j = (int)(t % ny);
    i = (int)(t / ny);
    if (img[c] != 0) return r;
    const long sj = nz, si = (long)ny * nz;
    bool has = false;
    if (j > 0 && img[c - sj] == 0) { r.v = 1; has = true; }
    if (j < ny - 1 && img[c + sj] == 0) has = true;
    if (k > 0 && img[c - 1] == 0) { r.w = 1; has = true; }
    if (k < nz - 1 && img[c + 1] == 0) has = true;
    if (i == 0) { u_west = 1; has = true; }
    if (i > 0 && img[c - si] == 0) { u_west = 1; has = true; }
    if (i == nx - 1) { u_out = 1; has = true; }
    if (i < nx - 1 && img[c + si] == 0) has = true;
    r.p = has ? 1 : 0;
    r.u = u_west + u_out;
    return r;
}

__device__ __forceinline__ int4 add4(int4 a, int4 b) { return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

__device__ __forceinline__ int4 shfl_up4(int4 v, int d) {
    return make_int4(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d),
                     __shfl_up_sync(0xffffffffu, v.z, d), __shfl_up_sync(0xffffffffu, v.w, d));
}

// exclusive block scan of int4 over GEO_THREADS threads; returns the
// exclusive prefix, `total` receives the block total
__device__ int4 block_exscan4(int4 v, int4 &total) {
    __shared__ int4 warp_tot[GEO_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int4 inc = v;
    for (int d = 1; d < 32; d <<= 1) {
        int4 o = shfl_up4(inc, d);
        if (lane >= d) inc = add4(inc, o);
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int4 run = make_int4(0, 0, 0, 0);
        for (int q = 0; q < GEO_THREADS / 32; ++q) {
            int4 tq = warp_tot[q];
            warp_tot[q] = run;
            run = add4(run, tq);
        }
        total = run;  // valid in thread 0 only
    }
    __syncthreads();
    int4 base = warp_tot[wid];
    int4 ex = add4(base, make_int4(inc.x - v.x, inc.y - v.y, inc.z - v.z, inc.w - v.w));
    return ex;
}

__global__ void k_count(const uint8_t *__restrict__ img, int nx, int ny, int nz, int4 *__restrict__ blk) {
    const long N = (long)nx * ny * nz;
    const long base = (long)blockIdx.x * GEO_CELLS + threadIdx.x * 4;
    int4 s = make_int4(0, 0, 0, 0);
    for (int m = 0; m < 4; ++m) {
        long c = base + m;
        if (c < N) {
            int i, j, k, uw, uo;
            CellCounts cc = cell_counts(img, nx, ny, nz, c, i, j, k, uw, uo);
            s = add4(s, make_int4(cc.p, cc.u, cc.v, cc.w));
        }
    }
    int4 tot;
    __shared__ int4 tot_sh;
    block_exscan4(s, tot);
    if (threadIdx.x == 0) tot_sh = tot;
    __syncthreads();
    if (threadIdx.x == 0) blk[blockIdx.x] = tot_sh;
}

// single block: exclusive scan of the per-block totals, sequential over tiles
__global__ void k_scan_blocks(int4 *__restrict__ blk, int nblk, int4 *__restrict__ totals) {
    __shared__ int4 carry_sh;
    if (threadIdx.x == 0) carry_sh = make_int4(0, 0, 0, 0);
    __syncthreads();
    for (int b0 = 0; b0 < nblk; b0 += GEO_THREADS) {
        int b = b0 + threadIdx.x;
        int4 v = (b < nblk) ? blk[b] : make_int4(0, 0, 0, 0);
        int4 tot;
        int4 ex = block_exscan4(v, tot);
        __shared__ int4 tot_sh;
        if (threadIdx.x == 0) tot_sh = tot;
        __syncthreads();
        int4 carry = carry_sh;
        if (b < nblk) blk[b] = add4(carry, ex);
        __syncthreads();
        if (threadIdx.x == 0) carry_sh = add4(carry, tot_sh);
        __syncthreads();
    }
    if (threadIdx.x == 0) *totals = carry_sh;
}

__global__ void k_scatter(const uint8_t *__restrict__ img, int nx, int ny, int nz, const int4 *__restrict__ blk,
                          int *__restrict__ pmap, int *__restrict__ umap, int *__restrict__ vmap,
                          int *__restrict__ wmap, int *__restrict__ pcell, int *__restrict__ ucell,
                          int *__restrict__ vcell, int *__restrict__ wcell) {
    const long N = (long)nx * ny * nz;
    const long base = (long)blockIdx.x * GEO_CELLS + threadIdx.x * 4;
    CellCounts cc[4];
    int ii[4], jj[4], kk[4], uw[4], uo[4];
    int4 s = make_int4(0, 0, 0, 0);
    for (int m = 0; m < 4; ++m) {
        long c = base + m;
        if (c < N) {
            cc[m] = cell_counts(img, nx, ny, nz, c, ii[m], jj[m], kk[m], uw[m], uo[m]);
        } else {
            cc[m] = {0, 0, 0, 0};
            uw[m] = uo[m] = 0;
        }
        s = add4(s, make_int4(cc[m].p, cc[m].u, cc[m].v, cc[m].w));
    }
    int4 tot;
    int4 off = add4(block_exscan4(s, tot), blk[blockIdx.x]);
    const long plane = (long)ny * nz;
    for (int m = 0; m < 4; ++m) {
        long c = base + m;
        if (c >= N) break;
        if (cc[m].v) { vmap[c] = off.z; vcell[off.z] = (int)c; off.z++; }
        if (cc[m].w) { wmap[c] = off.w; wcell[off.w] = (int)c; off.w++; }
        if (uw[m]) {
            long uc = c;  // umap position (i, j, k) with the same i
            umap[uc] = off.y; ucell[off.y] = (int)uc; off.y++;
        }
        if (uo[m]) {
            long uc = (long)nx * plane + (long)jj[m] * nz + kk[m];  // (nx, j, k)
            umap[uc] = off.y; ucell[off.y] = (int)uc; off.y++;
        }
        if (cc[m].p) { pmap[c] = off.x; pcell[off.x] = (int)c; off.x++; }
    }
}

// Neighbour columns of the momentum systems: the node of the same map in each
// direction (src/NSBase.cxx:911-1046; z only when the image has nz > 1).
__global__ void k_nbr_mom(const int *__restrict__ map, int d0, int ny, int nz, const int *__restrict__ cell, int n,
                          int npad, int *__restrict__ nbr, int zdir) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        long c = cell[r];
        int k = (int)(c % nz), j = (int)((c / nz) % ny), i = (int)(c / ((long)ny * nz));
        const long si = (long)ny * nz, sj = nz;
        nbr[0 * (size_t)npad + r] = (i - 1 >= 0) ? map[c - si] : -1;
        nbr[1 * (size_t)npad + r] = (i + 1 < d0) ? map[c + si] : -1;
        nbr[2 * (size_t)npad + r] = (j - 1 >= 0) ? map[c - sj] : -1;
        nbr[3 * (size_t)npad + r] = (j + 1 < ny) ? map[c + sj] : -1;
        nbr[4 * (size_t)npad + r] = (zdir && k - 1 >= 0) ? map[c - 1] : -1;
        nbr[5 * (size_t)npad + r] = (zdir && k + 1 < nz) ? map[c + 1] : -1;
    }
}

// Neighbour columns of the pressure systems: neighbour cell node and the face
// node between them (src/NSBase.cxx:525-573).
__global__ void k_nbr_p(Grid g, const int *__restrict__ cell, int n, int npad, int *__restrict__ nbr) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        int i, j, k;
        g.ijk(cell[r], i, j, k);
        int nx = g.nx, ny = g.ny, nz = g.nz;
        nbr[0 * (size_t)npad + r] = (i > 0 && g.P(i - 1, j, k) > -1 && g.U(i, j, k) > -1) ? g.P(i - 1, j, k) : -1;
        nbr[1 * (size_t)npad + r] = (i < nx - 1 && g.P(i + 1, j, k) > -1 && g.U(i + 1, j, k) > -1) ? g.P(i + 1, j, k) : -1;
        nbr[2 * (size_t)npad + r] = (j > 0 && g.P(i, j - 1, k) > -1 && g.V(i, j, k) > -1) ? g.P(i, j - 1, k) : -1;
        nbr[3 * (size_t)npad + r] = (j < ny - 1 && g.P(i, j + 1, k) > -1 && g.V(i, j + 1, k) > -1) ? g.P(i, j + 1, k) : -1;
        nbr[4 * (size_t)npad + r] = (k > 0 && g.P(i, j, k - 1) > -1 && g.W(i, j, k) > -1) ? g.P(i, j, k - 1) : -1;
        nbr[5 * (size_t)npad + r] = (k < nz - 1 && g.P(i, j, k + 1) > -1 && g.W(i, j, k + 1) > -1) ? g.P(i, j, k + 1) : -1;
    }
}

// ---- host launchers -------------------------------------------------------
void launch_build_image(const uint8_t *raw, int rnx, int rny, int rnz, int dir, int border, int pv, uint8_t *img,
                        int nx, int ny, int nz, cudaStream_t st) {
    long N = (long)nx * ny * nz;
    int grid = (int)std::min<long>((N + 255) / 256, 152L * 64);
    count_launches(1); k_build_image<<<grid, 256, 0, st>>>(raw, rnx, rny, rnz, dir, border, (uint8_t)pv, img, nx, ny, nz);
}

void launch_index_build(const uint8_t *img, int nx, int ny, int nz, int4 *blk, int4 *totals, int *pmap, int *umap,
                        int *vmap, int *wmap, int *pcell, int *ucell, int *vcell, int *wcell, cudaStream_t st) {
    long N = (long)nx * ny * nz;
    int nblk = (int)((N + GEO_CELLS - 1) / GEO_CELLS);
    count_launches(1); k_count<<<nblk, GEO_THREADS, 0, st>>>(img, nx, ny, nz, blk);
    count_launches(1); k_scan_blocks<<<1, GEO_THREADS, 0, st>>>(blk, nblk, totals);
    count_launches(1); k_scatter<<<nblk, GEO_THREADS, 0, st>>>(img, nx, ny, nz, blk, pmap, umap, vmap, wmap, pcell, ucell, vcell, wcell);
}

int index_build_blocks(long ncells) { return (int)((ncells + GEO_CELLS - 1) / GEO_CELLS); }

void launch_nbr_mom(const int *map, int d0, int ny, int nz, const int *cell, int n, int npad, int *nbr, int zdir,
                    cudaStream_t st) {
    if (n <= 0) return;
    int grid = std::min((n + 255) / 256, 152 * 32);
    count_launches(1); k_nbr_mom<<<grid, 256, 0, st>>>(map, d0, ny, nz, cell, n, npad, nbr, zdir);
}

void launch_nbr_p(const Grid &g, const int *cell, int n, int npad, int *nbr, cudaStream_t st) {
    if (n <= 0) return;
    int grid = std::min((n + 255) / 256, 152 * 32);
    count_launches(1); k_nbr_p<<<grid, 256, 0, st>>>(g, cell, n, npad, nbr);
}

}  // namespace ns3d
