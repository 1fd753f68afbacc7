/* The DEM pre-pass of a coupled run (lake_catchment_smooth,
 * SW2D-EFDC.cu:2766-2827) as a device pass on caller-owned device arrays.
 *
 * The reference sweeps the raster row by row from the last (south) row to
 * the first, each row west to east, updating in place: a catchment cell on
 * the lake edge takes the mean of its two neighbours across the edge, and
 * reads the cells south and west of it after their own update.  Only cells
 * on the mask edge change.  Numbering the anti-diagonals d = (rows-1-r) + c,
 * a cell's south and west neighbours lie on d-1 and its north and east
 * neighbours on d+1, so the cells of one diagonal are independent and the
 * sweep is a wavefront: the edge cells are listed per diagonal (count, scan,
 * fill), then one CTA walks the diagonals in order with a barrier between
 * non-empty ones.  Every update is the reference's (a + b) / 2.0 on the
 * same operands, so the result is bit-identical to the sequential sweep.
 * Compiled with --fmad=false.
 */
#include "sw2d.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

namespace sw2d {
void set_error_message(const char* msg); /* sw2d_api.cu */
}

namespace {

constexpr double kRefNodata = -9999.0; /* the literal the reference compares against */

__device__ __forceinline__ bool lake_edge(const int* __restrict__ m, int R, int C, int r, int c) {
    if (r < 1 || r > R - 2 || c < 1 || c > C - 2) return false;
    const size_t k = (size_t)r * C + c;
    const int v = m[k];
    return v != 1 && (v != m[k - C] || v != m[k + C] || v != m[k - 1] || v != m[k + 1]);
}

__global__ void k_lake_count(const int* __restrict__ m, int R, int C, int* __restrict__ cnt) {
    const long long n = (long long)R * C;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(k / C), c = (int)(k - (long long)r * C);
        if (lake_edge(m, R, C, r, c)) atomicAdd(&cnt[(R - 1 - r) + c], 1);
    }
}

/* exclusive scan of n counts in place (one block of 1024 threads); cnt[n]
 * receives the total */
__global__ void __launch_bounds__(1024) k_lake_scan(int* cnt, int n) {
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int per = (n + 1023) / 1024, a = min(n, t * per), b = min(n, a + per);
    int s = 0;
    for (int k = a; k < b; k++) s += cnt[k];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) { /* inclusive scan of the chunk sums */
        const int v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = t ? part[t - 1] : 0;
    for (int k = a; k < b; k++) {
        const int v = cnt[k];
        cnt[k] = run;
        run += v;
    }
    if (t == 1023) cnt[n] = part[1023];
}

__global__ void k_lake_fill(const int* __restrict__ m, int R, int C, const int* __restrict__ start,
                            int* __restrict__ fill, int* __restrict__ list) {
    const long long n = (long long)R * C;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(k / C), c = (int)(k - (long long)r * C);
        if (!lake_edge(m, R, C, r, c)) continue;
        const int d = (R - 1 - r) + c;
        list[start[d] + atomicAdd(&fill[d], 1)] = (int)k;
    }
}

/* the wavefront: one CTA, diagonals in order; within a diagonal the cells
 * are independent (the order of the list does not matter) */
__global__ void __launch_bounds__(1024) k_lake_sweep(const int* __restrict__ m, int C, const int* __restrict__ start,
                                                     const int* __restrict__ list, int nd, double* z) {
    for (int d = 0; d < nd; d++) {
        const int a = start[d], b = start[d + 1];
        if (a == b) continue;
        for (int j = a + threadIdx.x; j < b; j += blockDim.x) {
            const size_t k = (size_t)list[j];
            const int v = m[k];
            /* across the edge with the row above, then below, then the
             * columns west and east: each test may overwrite the last
             * (SW2D-EFDC.cu:2790-2816) */
            if (v != m[k - C] && z[k + C] != kRefNodata) z[k] = (z[k - C] + z[k + C]) / 2.0;
            if (v != m[k + C] && z[k - C] != kRefNodata) z[k] = (z[k - C] + z[k + C]) / 2.0;
            if (v != m[k - 1] && z[k + 1] != kRefNodata) z[k] = (z[k - 1] + z[k + 1]) / 2.0;
            if (v != m[k + 1] && z[k - 1] != kRefNodata) z[k] = (z[k - 1] + z[k + 1]) / 2.0;
        }
        __syncthreads(); /* the diagonal's updates are read by the next one */
    }
}

int fail(int code, const char* what, cudaError_t e = cudaSuccess) {
    char buf[256];
    if (e != cudaSuccess)
        std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    else
        std::snprintf(buf, sizeof buf, "%s", what);
    sw2d::set_error_message(buf);
    return code;
}

} // namespace

extern "C" int sw2d_lake_catchment_smooth_device(int rows, int cols, const int* d_mask, double* d_dem,
                                                 void* stream) {
    if (!d_mask || !d_dem) return fail(SW2D_ERR_INVALID, "null argument");
    if (rows < 1 || cols < 1) return fail(SW2D_ERR_INVALID, "rows and cols must be >= 1");
    if ((long long)rows * cols > (1LL << 30)) return fail(SW2D_ERR_INVALID, "rows * cols above 2^30 cells");
    if (rows < 3 || cols < 3) return SW2D_OK; /* no interior cell: nothing changes */
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nd = rows + cols - 1;
    int* d_cnt = nullptr;
    int* d_list = nullptr;
    cudaError_t e = cudaMalloc(&d_cnt, sizeof(int) * (size_t)(2 * nd + 2));
    if (e != cudaSuccess) return fail(SW2D_ERR_NOMEM, "cudaMalloc", e);
    int* d_fill = d_cnt + nd + 1;
    int total = 0;
    const long long n = (long long)rows * cols;
    const int grid = (int)std::min<long long>((n + 255) / 256, 152 * 16);
    e = cudaMemsetAsync(d_cnt, 0, sizeof(int) * (size_t)(2 * nd + 2), s);
    if (e == cudaSuccess) {
        k_lake_count<<<grid, 256, 0, s>>>(d_mask, rows, cols, d_cnt);
        k_lake_scan<<<1, 1024, 0, s>>>(d_cnt, nd);
        e = cudaMemcpyAsync(&total, d_cnt + nd, sizeof(int), cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess && total > 0) {
        e = cudaMalloc(&d_list, sizeof(int) * (size_t)total);
        if (e == cudaSuccess) {
            k_lake_fill<<<grid, 256, 0, s>>>(d_mask, rows, cols, d_cnt, d_fill, d_list);
            k_lake_sweep<<<1, 1024, 0, s>>>(d_mask, cols, d_cnt, d_list, nd, d_dem);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
    }
    cudaFree(d_list);
    cudaFree(d_cnt);
    if (e != cudaSuccess) return fail(SW2D_ERR_CUDA, "lake-edge device pass", e);
    return SW2D_OK;
}
