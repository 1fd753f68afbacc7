/* State measure on caller-owned device arrays that allocates nothing
 * (declared in include/sw2d_noalloc.h).
 *
 * The kernel is the measuring half of the FP64 path's prime kernel (volume
 * of the active cells and the exact CFL face-speed maxima) over the
 * reference-orientation arrays, with the per-tile partial results in a
 * file-scope device array instead of a buffer the handle allocates.  Compiled
 * with --fmad=false like the FP64 step, so the face speeds round exactly as
 * the step's own.
 */
#include "sw2d.h"
#include "sw2d_noalloc.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

namespace sw2d {
void set_error_message(const char* msg); /* sw2d_api.cu: the message sw2d_last_error returns */
}

namespace {

constexpr int kTile = SW2D_NOALLOC_TILE;              /* 32 x 32 cells per CTA */
constexpr int kRowsPerThread = kTile / 8;             /* 256 threads = 32 x 8 */
constexpr int kMaxTiles = SW2D_NOALLOC_MAX_TILES;
constexpr int kSlots = 3;                             /* volume, x speed bits, y speed bits */
constexpr int kResult = kSlots * kMaxTiles;           /* volume * area, speed */
constexpr int kCounter = kResult + 2;                 /* tile-completion counter (low 32 bits) */
constexpr int kScratchDoubles = kCounter + 1;         /* 49,155 doubles = 393,240 bytes */

/* The scratch: kSlots partials per tile, the two results, the counter. */
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

static_assert(sizeof(double) * kScratchDoubles == 393240, "scratch size stated in sw2d_noalloc.h");

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

/* (|velocity| + sqrt(g hm)) / spacing as the FP64 step evaluates it; positive
 * binary64 values order like their bit patterns, so maxima are taken on bits */
__device__ __forceinline__ unsigned long long face_speed_bits(double q, double hm, double g, double rd) {
    const double vel = (q == 0.0) ? q : __ddiv_rn(q, hm);
    const double s = __dmul_rn(__dadd_rn(fabs(vel), __dsqrt_rn(__dmul_rn(g, hm))), rd);
    return (unsigned long long)__double_as_longlong(s);
}

__global__ void __launch_bounds__(256) k64_measure_noalloc(const double* __restrict__ dem,
                                                           const double* __restrict__ h,
                                                           const double* __restrict__ qx,
                                                           const double* __restrict__ qy, int R, int C,
                                                           double nodata, double th, double g, double rdx,
                                                           double rdy, double area, double* scratch) {
    __shared__ double sv[8];
    __shared__ unsigned long long sx[8], sy[8];
    __shared__ bool last;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    const int c = blockIdx.x * kTile + tx;
    double vol = 0.0;
    unsigned long long ux = 0ull, uy = 0ull;
#pragma unroll
    for (int k = 0; k < kRowsPerThread; k++) {
        const int r = blockIdx.y * kTile + ty + 8 * k;
        if (r >= R || c >= C) continue;
        const size_t i = (size_t)r * C + c;
        if (dem[i] == nodata) continue;
        const double hc = h[i];
        vol = __dadd_rn(vol, hc);
        if (r > 0 && dem[i - C] != nodata) { /* x face north of (r, c) */
            const double hm = __dmul_rn(0.50, __dadd_rn(hc, h[i - C]));
            if (hm >= th) {
                const unsigned long long b = face_speed_bits(qx[i], hm, g, rdx);
                ux = b > ux ? b : ux;
            }
        }
        if (c > 0 && dem[i - 1] != nodata) { /* y face west of (r, c) */
            const double hn = __dmul_rn(0.50, __dadd_rn(hc, h[i - 1]));
            if (hn >= th) {
                const unsigned long long b = face_speed_bits(qy[(size_t)r * (C + 1) + c], hn, g, rdy);
                uy = b > uy ? b : uy;
            }
        }
    }
    vol = warp_sum(vol);
    ux = warp_max_u64(ux);
    uy = warp_max_u64(uy);
    if (tx == 0) {
        sv[ty] = vol;
        sx[ty] = ux;
        sy[ty] = uy;
    }
    __syncthreads();
    const int nb = gridDim.x * gridDim.y;
    const int b = blockIdx.y * gridDim.x + blockIdx.x;
    if (tid == 0) {
        double v = 0.0;
        unsigned long long a = 0ull, w = 0ull;
        for (int k = 0; k < 8; k++) {
            v = __dadd_rn(v, sv[k]);
            a = sx[k] > a ? sx[k] : a;
            w = sy[k] > w ? sy[k] : w;
        }
        scratch[(size_t)kSlots * b + 0] = v;
        scratch[(size_t)kSlots * b + 1] = __longlong_as_double((long long)a);
        scratch[(size_t)kSlots * b + 2] = __longlong_as_double((long long)w);
        __threadfence();
        unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kCounter);
        last = (atomicAdd(counter, 1u) == (unsigned int)nb - 1u);
    }
    __syncthreads();
    if (!last) return;
    /* the last tile to finish combines the partials in a fixed order */
    __threadfence();
    double v = 0.0;
    unsigned long long a = 0ull, w = 0ull;
    for (int k = tid; k < nb; k += 256) {
        const volatile double* pk = scratch + (size_t)kSlots * k;
        v = __dadd_rn(v, pk[0]);
        const unsigned long long pa = (unsigned long long)__double_as_longlong(pk[1]);
        const unsigned long long pw = (unsigned long long)__double_as_longlong(pk[2]);
        a = pa > a ? pa : a;
        w = pw > w ? pw : w;
    }
    v = warp_sum(v);
    a = warp_max_u64(a);
    w = warp_max_u64(w);
    __syncthreads();
    if (tx == 0) {
        sv[ty] = v;
        sx[ty] = a;
        sy[ty] = w;
    }
    __syncthreads();
    if (tid == 0) {
        double vt = 0.0;
        unsigned long long at = 0ull, wt = 0ull;
        for (int k = 0; k < 8; k++) {
            vt = __dadd_rn(vt, sv[k]);
            at = sx[k] > at ? sx[k] : at;
            wt = sy[k] > wt ? sy[k] : wt;
        }
        scratch[kResult + 0] = __dmul_rn(vt, area);
        scratch[kResult + 1] =
            __dadd_rn(__longlong_as_double((long long)at), __longlong_as_double((long long)wt));
    }
}

int reject(int code, const char* msg) {
    sw2d::set_error_message(msg);
    return code;
}

int cuda_fail(const char* what, cudaError_t e) {
    char buf[256];
    std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    sw2d::set_error_message(buf);
    return SW2D_ERR_CUDA;
}

} // namespace

extern "C" int sw2d_measure_state_noalloc(const double* d_dem, const double* d_depth, const double* d_qx,
                                          const double* d_qy, int rows, int cols, double dx, double dy,
                                          double nodata, double th, double g, void* stream, double* volume_out,
                                          double* speed_out) {
    if (!d_dem || !d_depth || !d_qx || !d_qy || !volume_out || !speed_out)
        return reject(SW2D_ERR_INVALID, "null argument");
    if (rows < 1 || cols < 1) return reject(SW2D_ERR_INVALID, "rows and cols must be >= 1");
    if (!(dx > 0.0) || !(dy > 0.0) || !(th > 0.0) || !(g > 0.0))
        return reject(SW2D_ERR_INVALID, "dx, dy, th and g must be > 0");
    if (static_cast<long long>(rows) * cols > (1LL << 30))
        return reject(SW2D_ERR_INVALID, "rows * cols above 2^30 cells");
    const long long tiles_x = (static_cast<long long>(cols) + kTile - 1) / kTile;
    const long long tiles_y = (static_cast<long long>(rows) + kTile - 1) / kTile;
    if (tiles_x * tiles_y > kMaxTiles) {
        char buf[200];
        std::snprintf(buf, sizeof buf,
                      "raster %d x %d spans %lld tiles of 32 x 32 cells; the no-allocation measure holds at most "
                      "%d (its scratch is fixed at 393,240 bytes)",
                      rows, cols, tiles_x * tiles_y, kMaxTiles);
        return reject(SW2D_ERR_INVALID, buf);
    }
    /* The scratch array's device address belongs to the calling thread's
     * current context (one copy per device, and a fresh copy after
     * cudaDeviceReset or under another context), so it is looked up on every
     * call rather than cached.  The lookup allocates nothing; in a context
     * that has not used the library's device code yet it loads that code
     * first, which is this entry point's one-time set-up. */
    void* addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail("cudaGetSymbolAddress", e);
    double* scratch = static_cast<double*>(addr);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    /* the counter must be zero when the kernel starts */
    e = cudaMemsetAsync(scratch + kCounter, 0, sizeof(double), s);
    if (e != cudaSuccess) return cuda_fail("cudaMemsetAsync", e);
    const dim3 grid((unsigned)tiles_x, (unsigned)tiles_y), block(32, 8);
    k64_measure_noalloc<<<grid, block, 0, s>>>(d_dem, d_depth, d_qx, d_qy, rows, cols, nodata, th, g, 1.0 / dx,
                                                1.0 / dy, dx * dy, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("k64_measure_noalloc launch", e);
    double res[2];
    e = cudaMemcpyAsync(res, scratch + kResult, sizeof res, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync", e);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail("cudaStreamSynchronize", e);
    *volume_out = res[0];
    *speed_out = res[1];
    return SW2D_OK;
}
