// Allocation-free binomial current filter.
//
// tg_filter_noalloc runs the ntimes passes of apply_filter1_opt on three
// current arrays the caller already owns on the device. The context-based
// tg_filter ping-pongs through scratch arrays that tg_init allocates; some
// callers cannot make that allocation: a host that hands the whole device
// to its own memory pool (CUDA Fortran / OpenACC managed arrays in a Fortran
// main loop), or a caller issuing work while it must not synchronise the
// device (cudaMalloc can serialise against running work). For them the
// scratch is a fixed file-scope __device__ array, so this entry point calls
// no cudaMalloc, cudaFree or allocating library routine.
//
// Costs and limits, stated for users:
//  * every GPU that loads the library holds the array (3 x
//    TG_NOALLOC_MAX_CELLS floats, 15.7 MB) until the process exits;
//  * grids above TG_NOALLOC_MAX_CELLS cells (mx*my*mz) are rejected;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and keeps it for the
//    life of the process; make that first call before any stream capture.
//    A cudaDeviceReset of that device makes the kept address stale: the
//    entry point must not be called on a device after a reset;
//  * error text goes to the per-thread message of tg_last_error(NULL);
//  * all calls share the one array: calls that overlap on the GPU (two
//    streams, or two host threads) race on it. Every pass writes every
//    scratch cell it later reads, so nothing needs clearing between calls.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "tg_internal.cuh"

using namespace tg;

static __device__ __align__(256) float g_filter_scratch[3 * (size_t)TG_NOALLOC_MAX_CELLS];

namespace {
constexpr int kMaxDevices = 64;
float *g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;
thread_local char g_noalloc_err[256];

int noalloc_fail(int code, const char *msg) {
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "tg_filter_noalloc: %s", msg);
    tg_set_global_error(g_noalloc_err);
    return code;
}
}  // namespace

extern "C" int tg_filter_noalloc(int32_t dims, int32_t mx, int32_t my, int32_t mz, int32_t nghost,
                                 int32_t nghostz, const int32_t *periodic, int32_t ntimes, float *curx,
                                 float *cury, float *curz, void *stream) {
    if (dims != 2 && dims != 3) return noalloc_fail(TG_ERR_ARG, "dims must be 2 or 3");
    if (!periodic || !curx || !cury || !curz) return noalloc_fail(TG_ERR_ARG, "null argument");
    if (nghost != 5 && nghost != 7) return noalloc_fail(TG_ERR_ARG, "nghost must be 5 or 7");
    if (dims == 2 && (mz != 1 || nghostz != 5)) return noalloc_fail(TG_ERR_ARG, "2D needs mz = 1, nghostz = 5");
    if (dims == 3 && nghostz != nghost) return noalloc_fail(TG_ERR_ARG, "3D needs nghostz = nghost");
    if (ntimes < 0) return noalloc_fail(TG_ERR_ARG, "ntimes must be >= 0");
    if (mx < nghost + 2 || my < nghost + 2 || (dims == 3 && mz < nghostz + 2))
        return noalloc_fail(TG_ERR_ARG, "grid smaller than its ghost layers");
    const long long lot = (long long)mx * my * mz;
    if (lot > (long long)TG_NOALLOC_MAX_CELLS) {
        char m[160];
        snprintf(m, sizeof m, "grid of %lld cells exceeds the fixed scratch of %d cells", lot,
                 (int)TG_NOALLOC_MAX_CELLS);
        return noalloc_fail(TG_ERR_ARG, m);
    }
    if (ntimes == 0) return TG_OK;

    // device address of the scratch array, looked up once per device
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return noalloc_fail(TG_ERR_CUDA, "no current CUDA device");
    float *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_filter_scratch);
            if (e != cudaSuccess) return noalloc_fail(TG_ERR_CUDA, cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<float *>(p);
        }
        scratch = g_scratch_addr[dev];
    }

    Geom g;
    memset(&g, 0, sizeof g);
    g.dims = dims;
    g.mx = mx;
    g.my = my;
    g.mz = mz;
    g.ng = nghost;
    g.ngz = nghostz;
    g.lot = lot;
    g.sy = mx;
    g.sz = (long long)mx * my;
    for (int a = 0; a < 3; a++) g.per[a] = periodic[a] ? 1 : 0;
    if (dims == 2) g.per[2] = 0;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *cur[3] = {curx, cury, curz};
    float *tmp[3] = {scratch, scratch + TG_NOALLOC_MAX_CELLS, scratch + 2 * (size_t)TG_NOALLOC_MAX_CELLS};
    for (int n = 0; n < ntimes; n++) {
        const cudaError_t e = (n % 2 == 0) ? launch_filter_pass(g, cur, tmp, st) : launch_filter_pass(g, tmp, cur, st);
        if (e != cudaSuccess) return noalloc_fail(TG_ERR_CUDA, cudaGetErrorString(e));
    }
    if (ntimes % 2 == 1)
        for (int c = 0; c < 3; c++) {
            const cudaError_t e = cudaMemcpyAsync(cur[c], tmp[c], (size_t)lot * 4, cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return noalloc_fail(TG_ERR_CUDA, cudaGetErrorString(e));
        }
    return TG_OK;
}
