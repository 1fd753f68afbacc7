/* SW2D GB300 -- state measure that allocates no memory.
 *
 * No counterpart in the reference: SW2D-EFDC.cu has no library API and never
 * measures a state outside its own time loop.  The computation is the one the
 * FP64 path performs on its own buffers when it primes the clock (volume of
 * the active cells, SW2D-EFDC.cu init_inf :37-42 for "active", and the CFL
 * face-speed sum that sets the next iteration's length); this entry point
 * runs it on depth / discharge arrays that the CALLER owns in device memory.
 *
 * Who needs it.  A caller that keeps its SW2D state in its own device arrays
 * (an EFDC-side coupling driver, a served job admitted against a fixed HBM
 * budget) and wants the volume and the CFL speed of that state cannot let a
 * library allocate on its behalf: an allocation can fail or evict a
 * neighbour when the device is filled to its budget, and cudaFree waits for
 * the whole device, stalling the kernels the caller keeps in flight on other
 * streams.  This call makes no cudaMalloc, cudaFree or other allocating call.
 *
 * Scratch.  The per-tile partial results live in one file-scope device array
 * of the library, 393,240 bytes, so the raster may span at most
 * SW2D_NOALLOC_MAX_TILES tiles of 32 x 32 cells (4096 x 4096 cells, or any
 * rows x cols with ceil(rows/32) * ceil(cols/32) <= 16384); larger rasters are
 * rejected with SW2D_ERR_INVALID before anything is launched.  The partial
 * slots need no initial value (each is written before it is read); the
 * tile-completion counter must be zero when the kernel starts, and each call
 * clears it on `stream` before its launch.
 *
 * Rules for the caller.
 *  - Calls share the one scratch array per device: two calls in flight at the
 *    same time (from two host threads, on any streams) race and corrupt each
 *    other's results.  Serialise them.  A call returns only after `stream`
 *    has finished its work, so calls from one host thread never overlap.
 *  - The scratch address is per CUDA context: every call looks it up with
 *    cudaGetSymbolAddress in the calling thread's current context (the
 *    caller's current device), so a call after cudaDeviceReset, or under
 *    another context of the same device, uses that context's own copy.  The
 *    first call in a context may load the library's device code into it
 *    (the set-up); make that first call before any stream capture begins on
 *    the device.  Later lookups only read the address.
 *  - Every call copies its two results to the host and synchronizes `stream`
 *    before it returns.
 *  - The device used is the caller's current device; every array must live
 *    on it.  Rasters above 2^30 cells are rejected like the other entry
 *    points' (SW2D_ERR_INVALID).
 */
#ifndef SW2D_NOALLOC_H
#define SW2D_NOALLOC_H

#ifdef __cplusplus
extern "C" {
#endif

#define SW2D_NOALLOC_TILE 32
#define SW2D_NOALLOC_MAX_TILES 16384

/* Volume and CFL speed of a state held in caller-owned device memory, in the
 * reference orientation (the layouts sw2d_get_state returns):
 *   d_dem   rows*cols bed elevations; cells equal to `nodata` are inactive
 *   d_depth rows*cols depths
 *   d_qx    (rows+1)*cols x-face discharges (row r = face north of cell row r)
 *   d_qy    rows*(cols+1) y-face discharges (column c = face west of column c)
 * stream: a cudaStream_t (NULL = the legacy default stream).
 * volume_out (host): sum over active cells of depth * dx * dy, m3.
 * speed_out (host): max over interior x faces of (|u| + sqrt(g hm)) / dx plus
 *   the same over interior y faces with dy, over faces between two active
 *   cells whose mean depth hm is >= th, u = q / hm (0 when q == 0) -- the
 *   speed s of the CFL rule, bit-identical to the FP64 path's own value for
 *   the same state (sw2d_get_ledger's s_max one iteration later).
 * Returns SW2D_OK, SW2D_ERR_INVALID (null pointer, size out of range) or
 * SW2D_ERR_CUDA (message in sw2d_last_error). */
int sw2d_measure_state_noalloc(const double* d_dem, const double* d_depth, const double* d_qx, const double* d_qy,
                               int rows, int cols, double dx, double dy, double nodata, double th, double g,
                               void* stream, double* volume_out, double* speed_out);

#ifdef __cplusplus
}
#endif
#endif
