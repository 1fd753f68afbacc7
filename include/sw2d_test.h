/* sw2d_test.h -- test hooks of libsw2d (not for production use).
 *
 * The reference has no failure handling to mirror (SW2D-EFDC.cu checks no
 * CUDA error); these hooks let tests drive the library's own failure paths
 * without faulting or hanging a GPU.
 */
#ifndef SW2D_TEST_H
#define SW2D_TEST_H

#include "sw2d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* FP32 handles: with on = 1 the marching kernel issues none of its staged
 * (TMA) loads for this handle's raster, so every CTA's bounded wait for its
 * first block runs out (about 2^31 cycles), the CTA sets the timeout bit in
 * the scenario's status word and returns with nothing in flight, and the next
 * sw2d_step / sw2d_advance returns SW2D_ERR_TIMEOUT.  The CUDA context stays
 * usable; the handle's clock has then advanced without its state, so restore
 * a snapshot (or set the depth again) after turning the hook off.  FP64
 * handles: SW2D_ERR_STATE (their kernels stage through plain loads). */
int sw2d_test_stall_staging(sw2d_handle* h, int on);

#ifdef __cplusplus
}
#endif
#endif
