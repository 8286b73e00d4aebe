// Particle launchers of the GB300 TRISTAN-MP hot path (sm_103a); kernel
// templates in tg_particles.cuh, the tile kernels instantiated per
// (dims, order) in tg_tiles_d*o*.cu.
#include "tg_particles.cuh"

namespace tg {

extern template cudaError_t launch_tiles_o<2, 1>(const TileArgs &, bool, bool, bool, cudaStream_t, size_t);
extern template cudaError_t launch_tiles_o<2, 2>(const TileArgs &, bool, bool, bool, cudaStream_t, size_t);
extern template cudaError_t launch_tiles_o<2, 3>(const TileArgs &, bool, bool, bool, cudaStream_t, size_t);
extern template cudaError_t launch_tiles_o<3, 1>(const TileArgs &, bool, bool, bool, cudaStream_t, size_t);
extern template cudaError_t launch_tiles_o<3, 2>(const TileArgs &, bool, bool, bool, cudaStream_t, size_t);
extern template cudaError_t launch_tiles_o<3, 3>(const TileArgs &, bool, bool, bool, cudaStream_t, size_t);
extern template cudaError_t launch_tail_o<2, 1>(const TileArgs &, const long long *, bool, cudaStream_t);
extern template cudaError_t launch_tail_o<2, 2>(const TileArgs &, const long long *, bool, cudaStream_t);
extern template cudaError_t launch_tail_o<2, 3>(const TileArgs &, const long long *, bool, cudaStream_t);

// ---------------------------------------------------------------------------
// tile counting sort
// ---------------------------------------------------------------------------
__global__ void k_tile_count(Geom g, Species sp, const long long *count, int *hist) {
    const long long nmax = *count;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nmax;
         n += (long long)gridDim.x * blockDim.x) {
        const int cell = sp.cell[n];
        if (cell < 0) continue;
        int i, j, k;
        cell_ijk(g, cell, i, j, k);
        agg_inc(hist, tile_of(g, i, j, k));
    }
}

// exclusive scan of hist[0..n) into start[0..n]; total -> *total; clears
// hist and cursor. One block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_tiles(int *hist, int *start, int *cursor, int n, long long *total) {
    __shared__ int warp_sums[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < n; base += blockDim.x) {
        const int idx = base + threadIdx.x;
        int v = idx < n ? hist[idx] : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int ws = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += t;
            }
            warp_sums[lane] = ws;
        }
        __syncthreads();
        const int wprefix = wid > 0 ? warp_sums[wid - 1] : 0;
        if (idx < n) {
            start[idx] = carry + wprefix + incl - v;
            hist[idx] = 0;
            cursor[idx] = 0;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += wprefix + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        start[n] = carry;
        *total = carry;
    }
}

// The records are read in blocks of 32 x TG_SCATTER_STRIDE, transposed: the
// lanes of a warp take records TG_SCATTER_STRIDE apart, and a warp's lanes
// bound for one tile get consecutive slots there. A tile's consecutive
// records, the lanes of one warp in the tile kernel, so come from different
// cells even where a loader wrote each cell's particles side by side (the
// window's shared atomics then meet fewer same-address and bank conflicts).
__global__ void k_tile_scatter(Geom g, Species src, Species dst, const long long *count, const int *start,
                               int *cursor) {
    constexpr int S = TG_SCATTER_STRIDE, B = 32 * S;
    const long long nmax = *count;
    const long long mmax = (nmax + B - 1) / B * B;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < mmax;
         m += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(m % B);
        const long long n = m - q + (q & 31) * S + (q >> 5);
        if (n >= nmax) continue;
        const int cell = src.cell[n];
        if (cell < 0) continue;
        // the record is read before its slot is claimed, so the loads'
        // latency overlaps the atomic's round trip
        const float ox = src.ox[n], oy = src.oy[n], oz = src.oz[n];
        const float u = src.u[n], v = src.v[n], w = src.w[n], ch = src.ch[n];
        const int32_t ind = src.ind[n], proc = src.proc[n], spl = src.splitlev[n];
        int i, j, k;
        cell_ijk(g, cell, i, j, k);
        const int t = tile_of(g, i, j, k);
        const long long d = (long long)start[t] + agg_inc(cursor, t);
        dst.cell[d] = cell;
        dst.ox[d] = ox;
        dst.oy[d] = oy;
        dst.oz[d] = oz;
        dst.u[d] = u;
        dst.v[d] = v;
        dst.w[d] = w;
        dst.ch[d] = ch;
        dst.ind[d] = ind;
        dst.proc[d] = proc;
        dst.splitlev[d] = spl;
    }
}

// gather by permutation (stable per-cell reorder)
__global__ void k_gather(Species src, Species dst, const int *perm, long long count) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < count;
         n += (long long)gridDim.x * blockDim.x) {
        const long long m = perm[n];
        dst.cell[n] = src.cell[m];
        dst.ox[n] = src.ox[m];
        dst.oy[n] = src.oy[m];
        dst.oz[n] = src.oz[m];
        dst.u[n] = src.u[m];
        dst.v[n] = src.v[m];
        dst.w[n] = src.w[m];
        dst.ch[n] = src.ch[m];
        dst.ind[n] = src.ind[m];
        dst.proc[n] = src.proc[m];
        dst.splitlev[n] = src.splitlev[m];
    }
}

// reference reorder key celli = int(x) + int(y)*iy + int(z)*iz
// (code/particles.F90:421), with the index as payload
__global__ void k_reorder_keys(Geom g, Species sp, long long count, int *keys, int *idx) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < count;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        cell_ijk(g, sp.cell[n], i, j, k);
        const int kz = g.dims == 3 ? k : (int)sp.oz[n];
        const long long key = (long long)i + (long long)j * g.sy + (g.dims == 3 ? (long long)kz * g.sz : 0);
        keys[n] = (int)key;
        idx[n] = (int)n;
    }
}

// ---------------------------------------------------------------------------
// AoS (reference records) <-> SoA
// ---------------------------------------------------------------------------
struct AoS {
    float x, y, z, u, v, w, ch;
    int32_t ind, proc, splitlev;
};

// Records pass through shared memory, so the AoS side moves as contiguous
// 8-byte words: coalesced in device memory and across NVLink-C2C when the
// records are host memory read or written in place. Each CTA converts
// chunks of TG_AOS_CHUNK records (40 B each; a chunk is 1280 words).
#define TG_AOS_CHUNK 256
template <int DIM>
__global__ void __launch_bounds__(TG_AOS_CHUNK)
    k_aos_to_soa(Geom g, const AoS *in, Species sp, long long count, int *status) {
    __shared__ unsigned long long buf[TG_AOS_CHUNK * 5];
    for (long long c0 = blockIdx.x * (long long)TG_AOS_CHUNK; c0 < count;
         c0 += (long long)gridDim.x * TG_AOS_CHUNK) {
        const int nrec = (int)min((long long)TG_AOS_CHUNK, count - c0);
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(in + c0);
        for (int t = threadIdx.x; t < nrec * 5; t += TG_AOS_CHUNK) buf[t] = src[t];
        __syncthreads();
        if (threadIdx.x < nrec) {
            const long long n = c0 + threadIdx.x;
            const AoS p = *reinterpret_cast<const AoS *>(buf + 5 * threadIdx.x);
            int i, j, k;
            if (pos_cell<DIM>(g, p.x, p.y, p.z, i, j, k)) {
                store_pos<DIM>(g, sp, n, p.x, p.y, p.z, i, j, k);
            } else {
                atomicOr(status, ST_BOUNDS);
                sp.cell[n] = -1;
            }
            sp.u[n] = p.u;
            sp.v[n] = p.v;
            sp.w[n] = p.w;
            sp.ch[n] = p.ch;
            sp.ind[n] = p.ind;
            sp.proc[n] = p.proc;
            sp.splitlev[n] = p.splitlev;
        }
        __syncthreads();
    }
}

template <int DIM>
__global__ void __launch_bounds__(TG_AOS_CHUNK) k_soa_to_aos(Geom g, Species sp, AoS *out, long long count) {
    __shared__ unsigned long long buf[TG_AOS_CHUNK * 5];
    for (long long c0 = blockIdx.x * (long long)TG_AOS_CHUNK; c0 < count;
         c0 += (long long)gridDim.x * TG_AOS_CHUNK) {
        const int nrec = (int)min((long long)TG_AOS_CHUNK, count - c0);
        if (threadIdx.x < nrec) {
            const long long n = c0 + threadIdx.x;
            AoS p;
            load_pos<DIM>(g, sp, n, p.x, p.y, p.z);
            p.u = sp.u[n];
            p.v = sp.v[n];
            p.w = sp.w[n];
            p.ch = sp.ch[n];
            p.ind = sp.ind[n];
            p.proc = sp.proc[n];
            p.splitlev = sp.splitlev[n];
            *reinterpret_cast<AoS *>(buf + 5 * threadIdx.x) = p;
        }
        __syncthreads();
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(out + c0);
        for (int t = threadIdx.x; t < nrec * 5; t += TG_AOS_CHUNK) dst[t] = buf[t];
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int grid_for(long long n, int block) {
    long long b = (n + block - 1) / block;
    if (b < 1) b = 1;
    if (b > 152 * 16) b = 152 * 16;
    return (int)b;
}

cudaError_t launch_tiles(const TileArgs &a, bool fixed, bool push, bool deposit, cudaStream_t st) {
    const size_t smem = deposit ? tile_smem_bytes(a.g.dims, a.g.wcells, a.g.fwcells) : 0;
    const int d = a.g.dims, o = a.g.order;
    if (d == 2 && o == 1) return launch_tiles_o<2, 1>(a, fixed, push, deposit, st, smem);
    if (d == 2 && o == 2) return launch_tiles_o<2, 2>(a, fixed, push, deposit, st, smem);
    if (d == 2 && o == 3) return launch_tiles_o<2, 3>(a, fixed, push, deposit, st, smem);
    if (d == 3 && o == 1) return launch_tiles_o<3, 1>(a, fixed, push, deposit, st, smem);
    if (d == 3 && o == 2) return launch_tiles_o<3, 2>(a, fixed, push, deposit, st, smem);
    return launch_tiles_o<3, 3>(a, fixed, push, deposit, st, smem);
}

cudaError_t launch_tail(const TileArgs &a, const long long *count, bool fixed, cudaStream_t st) {
    if (a.g.dims != 2) return cudaErrorInvalidValue;  // injection is 2D only
    if (a.g.order == 1) return launch_tail_o<2, 1>(a, count, fixed, st);
    if (a.g.order == 2) return launch_tail_o<2, 2>(a, count, fixed, st);
    return launch_tail_o<2, 3>(a, count, fixed, st);
}

cudaError_t launch_push_flat(const Geom &g, const Params &P, const FieldPtrs &f, const Species &sp,
                             const long long *dcount, long long count, float qm, int *status, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    const int grid = grid_for(count, 256);
    const int d = g.dims, o = g.order;
    if (d == 2 && o == 1) k_push_flat<2, 1><<<grid, 256, 0, st>>>(g, P, f, sp, dcount, qm, status);
    else if (d == 2 && o == 2) k_push_flat<2, 2><<<grid, 256, 0, st>>>(g, P, f, sp, dcount, qm, status);
    else if (d == 2 && o == 3) k_push_flat<2, 3><<<grid, 256, 0, st>>>(g, P, f, sp, dcount, qm, status);
    else if (d == 3 && o == 1) k_push_flat<3, 1><<<grid, 256, 0, st>>>(g, P, f, sp, dcount, qm, status);
    else if (d == 3 && o == 2) k_push_flat<3, 2><<<grid, 256, 0, st>>>(g, P, f, sp, dcount, qm, status);
    else k_push_flat<3, 3><<<grid, 256, 0, st>>>(g, P, f, sp, dcount, qm, status);
    return cudaGetLastError();
}

cudaError_t launch_tile_count(const Geom &g, const Species &sp, const long long *count, long long hint, int *hist,
                              cudaStream_t st) {
    k_tile_count<<<grid_for(hint, 256), 256, 0, st>>>(g, sp, count, hist);
    return cudaGetLastError();
}

cudaError_t launch_scan(int *hist, int *start, int *cursor, int n, long long *total, cudaStream_t st) {
    k_scan_tiles<<<1, 1024, 0, st>>>(hist, start, cursor, n, total);
    return cudaGetLastError();
}

cudaError_t launch_scatter(const Geom &g, const Species &src, const Species &dst, const long long *count,
                           long long hint, const int *start, int *cursor, cudaStream_t st) {
    k_tile_scatter<<<grid_for(hint, 256), 256, 0, st>>>(g, src, dst, count, start, cursor);
    return cudaGetLastError();
}

cudaError_t launch_gather(const Species &src, const Species &dst, const int *perm, long long count,
                          cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    k_gather<<<grid_for(count, 256), 256, 0, st>>>(src, dst, perm, count);
    return cudaGetLastError();
}

cudaError_t launch_reorder_keys(const Geom &g, const Species &sp, long long count, int *keys, int *idx,
                                cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    k_reorder_keys<<<grid_for(count, 256), 256, 0, st>>>(g, sp, count, keys, idx);
    return cudaGetLastError();
}

cudaError_t launch_aos_to_soa(const Geom &g, const void *in, const Species &sp, long long count, int *status,
                              cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    if ((uintptr_t)in & 7) return cudaErrorMisalignedAddress;  // records move as 8-byte words
    if (g.dims == 3)
        k_aos_to_soa<3><<<grid_for(count, 256), 256, 0, st>>>(g, (const AoS *)in, sp, count, status);
    else
        k_aos_to_soa<2><<<grid_for(count, 256), 256, 0, st>>>(g, (const AoS *)in, sp, count, status);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const Geom &g, const Species &sp, void *out, long long count, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    if ((uintptr_t)out & 7) return cudaErrorMisalignedAddress;  // records move as 8-byte words
    if (g.dims == 3) k_soa_to_aos<3><<<grid_for(count, 256), 256, 0, st>>>(g, sp, (AoS *)out, count);
    else k_soa_to_aos<2><<<grid_for(count, 256), 256, 0, st>>>(g, sp, (AoS *)out, count);
    return cudaGetLastError();
}

}  // namespace tg
