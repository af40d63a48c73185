// hmec_sort.cuh -- the deterministic counting sort of markers by half cell,
// shared by the context path (k_p2g.cu) and the allocation-free path
// (k_p2g_static.cu).
//
// The node gathers of sections a3-a4 (cpp/h_mec_rsf_v9.cpp:435-583) sum
// over each half cell's markers in the sorted order, so that order must be a
// function of the input alone: within a half cell, markers in increasing
// index.  The sort:
//   1. k_keys: the half-cell key of every marker (the reference's cell
//      indices, bit-exact) and a warp-aggregated histogram of the keys;
//   2. k_scan1-3: exclusive scan of the counts -> segment starts (and the
//      scatter cursors);
//   3. k_scatter: warp-aggregated atomic scatter (each segment receives the
//      right markers, in arrival order);
//   4. k_segsort: each segment of at most SEG_SHORT markers is put in index
//      order by one thread; a longer segment (markers that cluster, or many
//      markers clamped into an edge cell) only raises the `long` flag;
//   5. k_radix_sort, gated by that flag: a stable LSD radix sort of all
//      (key, marker) pairs in one cooperative launch, which rebuilds the whole
//      permutation in (key, index) order in O(n) whatever the segment lengths.
// Steps 4 and 5 give the same permutation, so the results do not depend on
// which one ran.
#pragma once

#include <cooperative_groups.h>

#include "hmec_internal.cuh"

namespace hsort {
// internal linkage: every translation unit that sorts gets its own kernels
namespace {

namespace cgs = cooperative_groups;

constexpr int SEG_SHORT = 64;  // longest segment k_segsort orders itself

// Half-cell key of a marker: (hc, hr) = (2 jb + (jP - jb), 2 ib + (iP - ib)),
// key = hc * 2(Ny-1) + hr.  iP - ib and jP - jb are 0 or 1 by the monotone
// clamp; the guard only keeps a corrupted index in range.
__device__ __forceinline__ int half_key(const MarkerCells& c, const Geo& g, int* status) {
    int di = c.iP - c.ib, dj = c.jP - c.jb;
    if (di < 0 || di > 1 || dj < 0 || dj > 1) {
        if (status) atomicOr(status, HMEC_DEV_BOUNDS);
        di = di < 0 ? 0 : (di > 1 ? 1 : di);
        dj = dj < 0 ? 0 : (dj > 1 ? 1 : dj);
    }
    return (2 * c.jb + dj) * (2 * (g.Ny - 1)) + 2 * c.ib + di;
}

// Keys in marker order and their histogram (one atomic per distinct key in a warp).
__global__ void k_keys(const double* __restrict__ xm, const double* __restrict__ ym, int64_t n, Geo g,
                       int32_t* __restrict__ key, int32_t* __restrict__ count, int* status) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int k = -1;
    if (m < n) {
        k = half_key(marker_cells(xm[m], ym[m], g), g, status);
        key[m] = k;
    }
    const unsigned active = __ballot_sync(0xffffffffu, k >= 0);
    if (k >= 0) {
        const unsigned peers = __match_any_sync(active, k);
        if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&count[k], __popc(peers));
    }
}

// Exclusive scan of n counts in three phases: block scans of 2048 (Blelloch),
// the scan of the block totals (part[nparts] receives the total), the add.
__global__ void k_scan1(const int32_t* __restrict__ in, int n, int32_t* __restrict__ out, int32_t* __restrict__ part) {
    __shared__ int32_t sh[2048];
    const int base = blockIdx.x * 2048;
    const int t = threadIdx.x;
    sh[t] = (base + t < n) ? in[base + t] : 0;
    sh[t + 1024] = (base + t + 1024 < n) ? in[base + t + 1024] : 0;
    __syncthreads();
    for (int d = 1; d < 2048; d <<= 1) {
        const int idx = (t + 1) * d * 2 - 1;
        if (idx < 2048) sh[idx] += sh[idx - d];
        __syncthreads();
    }
    if (t == 0) {
        part[blockIdx.x] = sh[2047];
        sh[2047] = 0;
    }
    __syncthreads();
    for (int d = 1024; d >= 1; d >>= 1) {
        const int idx = (t + 1) * d * 2 - 1;
        if (idx < 2048) {
            const int32_t v = sh[idx - d];
            sh[idx - d] = sh[idx];
            sh[idx] += v;
        }
        __syncthreads();
    }
    if (base + t < n) out[base + t] = sh[t];
    if (base + t + 1024 < n) out[base + t + 1024] = sh[t + 1024];
}

__global__ void k_scan2(int32_t* __restrict__ part, int nparts) {
    // one block of 1024 threads: carry over chunks of 1024 block totals
    __shared__ int32_t sh[1024];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < nparts; c0 += 1024) {
        const int t = threadIdx.x;
        const int32_t v = (c0 + t < nparts) ? part[c0 + t] : 0;
        sh[t] = v;
        __syncthreads();
        for (int d = 1; d < 1024; d <<= 1) {  // Hillis-Steele inclusive scan
            const int32_t a = (t >= d) ? sh[t - d] : 0;
            __syncthreads();
            sh[t] += a;
            __syncthreads();
        }
        if (c0 + t < nparts) part[c0 + t] = carry + sh[t] - v;
        __syncthreads();
        if (t == 0) carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[nparts] = carry;
}

// out += the block offsets; cursor (if set) receives a copy (the scatter's cursors)
__global__ void k_scan3(int32_t* __restrict__ out, int n, const int32_t* __restrict__ part, int32_t* cursor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int32_t v = out[i] + part[i / 2048];
        out[i] = v;
        if (cursor) cursor[i] = v;
    }
}

__global__ void k_scatter(const int32_t* __restrict__ key, int64_t n, int32_t* __restrict__ cursor,
                          int32_t* __restrict__ perm) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = (m < n) ? key[m] : -1;
    const unsigned active = __ballot_sync(0xffffffffu, k >= 0);
    if (k >= 0) {
        const unsigned peers = __match_any_sync(active, k);
        const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&cursor[k], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        perm[base + __popc(peers & ((1u << lane) - 1u))] = (int32_t)m;
    }
}

// Segments of at most SEG_SHORT markers into index order (insertion sort,
// one thread each); a longer segment sets *long_flag and is left to
// k_radix_sort.
__global__ void k_segsort(const int32_t* __restrict__ start, int nseg, int32_t* __restrict__ perm, int* long_flag) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int b = start[s], e = start[s + 1];
    if (e - b > SEG_SHORT) {
        *long_flag = 1;
        return;
    }
    for (int a = b + 1; a < e; a++) {
        const int v = perm[a];
        int q = a;
        while (q > b && perm[q - 1] > v) {
            perm[q] = perm[q - 1];
            q--;
        }
        perm[q] = v;
    }
}

// ------------------------------------------------------------ radix sort
// Stable LSD radix sort of the keys (RS_BITS per pass) carrying the marker
// index, as one cooperative launch; grid barriers separate each pass's
// tile histograms, their scan and the scatter.  A tile is RS_BS consecutive
// elements, one per thread; an element's rank among the equal digits of its
// tile comes from warp matching and per-warp digit counts, so the tile keeps
// the input order and so does every pass.
constexpr int RS_BS = 512;
constexpr int RS_BITS = 8;
constexpr int RS_BINS = 1 << RS_BITS;
constexpr int RS_WARPS = RS_BS / 32;
static_assert(RS_BINS <= RS_BS, "one thread per digit for the warp prefix");

constexpr int RS_MAXPASS = 4;  // 32-bit keys
struct RadixArgs {
    int64_t n;
    int passes;
    // pass p reads keys kin[p] and marker indices vin[p] (null: the element's
    // own index, the first pass) and writes kout[p] (not on the last pass)
    // and vout[p]; the host chains them so that the last pass writes the
    // permutation
    const int32_t* kin[RS_MAXPASS];
    const int32_t* vin[RS_MAXPASS];
    int32_t* kout[RS_MAXPASS];
    int32_t* vout[RS_MAXPASS];
    int32_t* hist;        // RS_BINS * ntiles digit counts, scanned in place
    int32_t* part;        // one partial sum per block
    const int* gate;      // the sort runs only when *gate != 0
};

// Bytes of scratch the radix sort needs beyond key0 and perm: two key
// buffers, one index buffer, the histograms and the block partials.
__host__ __device__ __forceinline__ size_t radix_scratch_ints(int64_t n, int max_blocks) {
    const int64_t ntiles = (n + RS_BS - 1) / RS_BS;
    return (size_t)(3 * n + RS_BINS * ntiles + max_blocks + 16);
}

// Sum of v over the block (every thread gets it).
__device__ __forceinline__ int block_sum_i(int v, int* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    int s = 0;
    for (int w = 0; w < RS_WARPS; w++) s += sh[w];
    return s;
}

// Exclusive prefix of v over the block's threads in thread order; *total gets the sum.
__device__ __forceinline__ int block_exscan_i(int v, int* sh, int* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    __syncthreads();
    if (lane == 31) sh[warp] = inc;
    __syncthreads();
    int off = 0, tot = 0;
    for (int w = 0; w < RS_WARPS; w++) {
        const int s = sh[w];
        if (w < warp) off += s;
        tot += s;
    }
    *total = tot;
    return off + inc - v;
}

// Digit d of this thread's element (-1: past the end) and its rank among the
// tile's elements of the same digit; tot[d] receives the tile's count of d.
__device__ __forceinline__ int tile_rank(int d, int (*wcnt)[RS_BINS], int* tot) {
    for (int q = threadIdx.x; q < RS_WARPS * RS_BINS; q += RS_BS) (&wcnt[0][0])[q] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rw = __popc(peers & ((1u << lane) - 1u));
    if (d >= 0 && rw == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (threadIdx.x < RS_BINS) {
        int acc = 0;
        for (int w = 0; w < RS_WARPS; w++) {
            const int v = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = acc;
            acc += v;
        }
        tot[threadIdx.x] = acc;
    }
    __syncthreads();
    return d >= 0 ? wcnt[warp][d] + rw : 0;
}

__global__ void __launch_bounds__(RS_BS) k_radix_sort(RadixArgs a) {
    if (a.gate && !*a.gate) return;  // written before this launch: uniform over the grid
    cgs::grid_group grid = cgs::this_grid();
    __shared__ int wcnt[RS_WARPS][RS_BINS];
    __shared__ int tot[RS_BINS];
    __shared__ int sh[RS_WARPS];
    const int64_t n = a.n;
    const int ntiles = (int)((n + RS_BS - 1) / RS_BS);
    const int64_t M = (int64_t)RS_BINS * ntiles;
    for (int p = 0; p < a.passes; p++) {
        const int shift = p * RS_BITS;
        const int32_t* kin = a.kin[p];
        const int32_t* vin = a.vin[p];
        int32_t* kout = a.kout[p];
        int32_t* vout = a.vout[p];
        const bool last = p == a.passes - 1;
        // tile histograms, digit-major: hist[d * ntiles + tile]
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const int64_t e = (int64_t)tile * RS_BS + threadIdx.x;
            const int d = e < n ? (kin[e] >> shift) & (RS_BINS - 1) : -1;
            tile_rank(d, wcnt, tot);
            if (threadIdx.x < RS_BINS) a.hist[(size_t)threadIdx.x * ntiles + tile] = tot[threadIdx.x];
            __syncthreads();
        }
        grid.sync();
        // exclusive scan of hist in place: each block a contiguous chunk
        {
            const int64_t chunk = (M + gridDim.x - 1) / gridDim.x;
            const int64_t c0 = (int64_t)blockIdx.x * chunk, c1 = c0 + chunk < M ? c0 + chunk : M;
            int s = 0;
            for (int64_t q = c0 + threadIdx.x; q < c1; q += RS_BS) s += a.hist[q];
            s = block_sum_i(s, sh);
            if (threadIdx.x == 0) a.part[blockIdx.x] = s;
            grid.sync();
            int off = 0;
            for (int b = threadIdx.x; b < (int)blockIdx.x; b += RS_BS) off += a.part[b];
            off = block_sum_i(off, sh);
            for (int64_t q0 = c0; q0 < c1; q0 += RS_BS) {
                const int64_t q = q0 + threadIdx.x;
                const int v = q < c1 ? a.hist[q] : 0;
                int t = 0;
                const int ex = block_exscan_i(v, sh, &t);
                if (q < c1) a.hist[q] = off + ex;
                off += t;
            }
        }
        grid.sync();
        // stable scatter
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const int64_t e = (int64_t)tile * RS_BS + threadIdx.x;
            int k = 0, v = 0, d = -1;
            if (e < n) {
                k = kin[e];
                v = vin ? vin[e] : (int)e;
                d = (k >> shift) & (RS_BINS - 1);
            }
            const int r = tile_rank(d, wcnt, tot);
            if (d >= 0) {
                const int pos = a.hist[(size_t)d * ntiles + tile] + r;
                vout[pos] = v;
                if (!last) kout[pos] = k;
            }
            __syncthreads();
        }
        grid.sync();
    }
}

// Buffers of the sort.  key: keys in marker order (k_keys); count: nh+1
// ints, zero on entry; start: nh+2; fill: nh+1; part: scan partials
// ((nh+1+2047)/2048 + 1); perm: n; long_flag: one int; radix: at least
// radix_scratch_ints(n, max_blocks) ints.
struct SortBufs {
    int32_t *key, *count, *start, *fill, *part, *perm;
    int* long_flag;
    int32_t* radix;
    int bs = 256;  // threads per block of the scatter
};

// Co-resident blocks of k_radix_sort (cached per process; one GPU type).
inline cudaError_t radix_grid(int* blocks) {
    static int cached = 0;
    if (!cached) {
        int dev = 0, nsm = 0, per_sm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_radix_sort, RS_BS, 0);
        if (e != cudaSuccess) return e;
        cached = per_sm * nsm > 0 ? per_sm * nsm : 1;
    }
    *blocks = cached;
    return cudaSuccess;
}

// Steps 2-5 on stream s, after k_keys filled key and count.  nh: number of
// half cells.  *launches is advanced by the kernels launched.
inline cudaError_t sort_by_half_cell(cudaStream_t s, const SortBufs& b, int64_t n, int nh, int64_t* launches) {
    const int ns = nh + 1;
    const int nparts = (ns + 2047) / 2048;
    k_scan1<<<nparts, 1024, 0, s>>>(b.count, ns, b.start, b.part);
    k_scan2<<<1, 1024, 0, s>>>(b.part, nparts);
    k_scan3<<<nblocks(ns, 256), 256, 0, s>>>(b.start, ns, b.part, b.fill);
    const int bs = b.bs > 0 ? b.bs : 256;
    k_scatter<<<nblocks(n, bs), bs, 0, s>>>(b.key, n, b.fill, b.perm);
    cudaError_t e = cudaMemsetAsync(b.long_flag, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    k_segsort<<<nblocks(nh, 128), 128, 0, s>>>(b.start, nh, b.perm, b.long_flag);
    int grid = 1;
    e = radix_grid(&grid);
    if (e != cudaSuccess) return e;
    const int ntiles = (int)((n + RS_BS - 1) / RS_BS);
    grid = grid < ntiles ? grid : (ntiles > 0 ? ntiles : 1);
    int nbits = 1;
    while (nbits < 31 && (1LL << nbits) < (long long)nh) nbits++;
    RadixArgs r;
    r.n = n;
    r.passes = (nbits + RS_BITS - 1) / RS_BITS;
    int32_t* kbuf[2] = {b.radix, b.radix + n};
    int32_t* vbuf[2] = {b.perm, b.radix + 2 * n};
    for (int p = 0; p < RS_MAXPASS; p++) {
        r.kout[p] = kbuf[p % 2];
        r.vout[p] = vbuf[((r.passes - 1 - p) % 2 + 2) % 2];  // the last pass writes perm
        r.kin[p] = p == 0 ? b.key : r.kout[p - 1];
        r.vin[p] = p == 0 ? nullptr : r.vout[p - 1];
    }
    r.hist = b.radix + 3 * n;
    r.part = r.hist + (size_t)RS_BINS * ntiles;
    r.gate = b.long_flag;
    void* args[] = {&r};
    e = cudaLaunchCooperativeKernel((const void*)k_radix_sort, dim3(grid), dim3(RS_BS), args, 0, s);
    if (launches) *launches += 7;
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace
}  // namespace hsort
