// noalloc.cu -- a BiCGSTAB entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool or a host that pre-reserves all device memory at
// start-up, callers that must not synchronize the device through an
// allocation, and embedded/real-time hosts that forbid allocation after
// initialisation.  ns3d_bicgstab_noalloc serves them: the caller passes the
// system (device pointers) and the vectors; every work vector, the chunk
// partials, the solver state and the loop kernel's grid barrier live in one
// file-scope device array of fixed size, kScratchRows rows (65536), declared
// below.  Every GPU that loads the
// library holds that array (about 4.5 MiB) until the process exits.
//
// Host code cannot use the array's name as a device address (it names a
// host-side stand-in), so the first call on each device looks the address up
// with cudaGetSymbolAddress while that device is current, checks the result
// and caches it.  Under CUDA's default lazy module loading this lookup is
// also what places the array (and this module's code) on the device, so the
// first call should come before the host reserves the rest of the device's
// memory, and before any stream capture.
// Every call shares the one array and overwrites it: calls that overlap on
// the GPU (two streams, two host threads) race, so serialize them.
#include <cstring>
#include <mutex>

#include "device.cuh"
#include "kernels.h"
#include "../../include/ns3d_capi.h"

namespace ns3d {
namespace {

constexpr int kScratchRows = 1 << 16;
constexpr int kScratchChunks = kScratchRows / CH;
constexpr int kVectors = 9;  // r, r0, p, v, y, s, z, t, invdiag
constexpr size_t kVecBytes = (size_t)kVectors * kScratchRows * sizeof(double);
constexpr size_t kPartBytes = (size_t)5 * kScratchChunks * sizeof(double);
constexpr size_t kStateOffset = kVecBytes + kPartBytes;
constexpr size_t kBarOffset = kStateOffset + 256;
constexpr size_t kScratchBytes = kBarOffset + 512;
static_assert(sizeof(KState) <= 256 && sizeof(GridBar) <= 512, "scratch layout");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_addr[kMaxDevices] = {nullptr};

// device address of the scratch array for the current device
int scratch_address(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return NS3D_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return NS3D_ERR_CUDA;
        g_addr[dev] = p;
    }
    *out = (unsigned char *)g_addr[dev];
    return NS3D_OK;
}

// Jacobi inverse diagonal (1/a_rr, or 1 for a zero diagonal)
__global__ void k_noalloc_invdiag(const double *__restrict__ diag, int n, double *__restrict__ inv) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const double d = diag[r];
        inv[r] = (d != 0.0) ? 1.0 / d : 1.0;
    }
}

// messages are static strings: reporting an error allocates nothing either
thread_local const char *g_noalloc_err = "";

int fail(int code, const char *msg) {
    g_noalloc_err = msg;
    return code;
}

}  // namespace
}  // namespace ns3d

using namespace ns3d;

extern "C" NS3D_API const char *ns3d_noalloc_last_error(void) { return g_noalloc_err; }

extern "C" NS3D_API int ns3d_bicgstab_noalloc(const double *coef, const int32_t *nbr, const double *rhs, double *x,
                                              int32_t n, int32_t npad, double tol, int32_t maxit, void *stream,
                                              ns3d_solve_info *info) {
    g_noalloc_err = "";  // the text describes this call's failure only
    if (!coef || !nbr || !rhs || !x || !info) return fail(NS3D_ERR_ARG, "NULL argument");
    if (n < 0 || maxit <= 0 || !(tol >= 0)) return fail(NS3D_ERR_ARG, "bad size, tolerance or iteration cap");
    if (n > kScratchRows) return fail(NS3D_ERR_ARG, "system larger than the 65536-row scratch of this entry point");
    if (npad < n || npad % CH != 0) return fail(NS3D_ERR_ARG, "npad must be >= n and a multiple of 1024");
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 0) {  // nothing to solve: reported like a zero right-hand side
        info->iterations = maxit;
        info->info = NS3D_SUCCESS;
        info->error = tol;
        return NS3D_OK;
    }
    unsigned char *base = nullptr;
    int rc = scratch_address(&base);
    if (rc != NS3D_OK) return fail(rc, "cudaGetSymbolAddress failed for the scratch array");
    double *vec = (double *)base;
    double *part = (double *)(base + kVecBytes);
    KState *dst = (KState *)(base + kStateOffset);
    GridBar *bar = (GridBar *)(base + kBarOffset);
    const int nchunks = (n + CH - 1) / CH;

    KSetArg set;
    std::memset(&set, 0, sizeof set);
    set.nsys = 1;
    set.total_chunks = nchunks;
    KSys &hs = set.sys[0];
    hs.n = n;
    hs.npad = npad;
    hs.nchunks = nchunks;
    hs.chunk_begin = 0;
    double *invdiag = vec + (size_t)8 * kScratchRows;
    hs.coef = coef;
    hs.nbr = nbr;
    hs.invdiag = invdiag;
    hs.b = rhs;
    hs.x = x;
    double **ws[8] = {&hs.r, &hs.r0, &hs.p, &hs.v, &hs.y, &hs.s, &hs.z, &hs.t};
    for (int i = 0; i < 8; ++i) *ws[i] = vec + (size_t)i * kScratchRows;
    hs.part = part;
    hs.st = dst;
    KState k0;
    std::memset(&k0, 0, sizeof k0);
    k0.tol = tol;
    k0.maxit = maxit;

    auto ok = [](cudaError_t e) { return e == cudaSuccess; };
    // the scratch keeps the previous call's contents: state, counter and the
    // inverse diagonal are rewritten here, p and v are zeroed by the init
    // kernels; the system's pointers travel as a kernel argument
    if (!ok(cudaMemcpyAsync(dst, &k0, sizeof k0, cudaMemcpyHostToDevice, st)) ||
        !ok(cudaMemsetAsync(invdiag, 0, (size_t)nchunks * CH * sizeof(double), st)))
        return fail(NS3D_ERR_CUDA, "scratch set-up copy failed");
    k_noalloc_invdiag<<<std::max(1, std::min((n + 255) / 256, 1024)), 256, 0, st>>>(coef, n, invdiag);
    count_launches(1);
    launch_krylov_init(set, st);
    const long cap = 2L * maxit + 64;
    long issued = 0;
    int work_before = 0, bar_err = 0;
    bool launched = false;
    KState h;
    while (true) {
        if (!ok(cudaMemcpyAsync(&h, dst, sizeof h, cudaMemcpyDeviceToHost, st)) ||
            !ok(cudaMemcpyAsync(&bar_err, &bar->err, sizeof bar_err, cudaMemcpyDeviceToHost, st)) ||
            !ok(cudaStreamSynchronize(st)))
            return fail(NS3D_ERR_CUDA, "CUDA error while solving (see cudaGetLastError)");
        if (launched && bar_err) return fail(NS3D_ERR_TIMEOUT, "BiCGSTAB loop kernel: a grid barrier timed out");
        if (h.done) break;
        if (launched && h.work == work_before && !h.paused)
            return fail(NS3D_ERR_TIMEOUT, "BiCGSTAB loop kernel made no progress");
        issued += h.work - work_before;
        work_before = h.work;
        if (issued >= cap) return fail(NS3D_ERR_TIMEOUT, "BiCGSTAB exceeded its iteration bound");
        if (h.paused) launch_krylov_restart(set, st);
        if (!ok(launch_krylov_loop(set, bar, nullptr, (int)(cap - issued), st)))
            return fail(NS3D_ERR_CUDA, "cooperative launch of the BiCGSTAB loop kernel failed");
        launched = true;
    }
    info->iterations = h.iter;
    info->info = h.info;
    info->error = h.error;
    return NS3D_OK;
}
