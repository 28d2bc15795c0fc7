/*
 * libshocks_check.so: the bounds-check build of libshocks (-DSHOCKS_BOUNDS_CHECK).
 *
 * Same sources and the same C ABI as libshocks.so (include/shocks.h), plus the
 * two entry points below. In this build every index into a kernel's
 * shared-memory window arrays, stage storage and state arrays is checked
 * against the bounds of its array; a violation is recorded in a device log
 * (first violation per translation unit: block, thread, element offset from
 * the array start, array extent), the access goes to a sink word instead, and
 * shk_plan_status reports ERR_BOUNDS (4) beside the plan's own status bits.
 * Nothing traps or asserts. The product library has none of this.
 *
 * No counterpart in the reference: these are test instruments, standing in
 * for a memory checker that is not available on the target machines.
 */
#ifndef SHOCKS_CHECK_H
#define SHOCKS_CHECK_H

#include <stdint.h>

#include "shocks.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Synchronises the device and reads the bounds logs of every translation
 * unit: *flag = 1 if an out-of-bounds index was recorded since the last
 * reset, with the first recorded block, thread, offset and extent (each
 * output may be NULL). reset != 0 clears the logs after reading them. */
int shk_check_bounds(int32_t reset, int32_t* flag, int32_t* block, int32_t* thread,
                     int64_t* offset, int64_t* extent);

/* Test hook: makes the window loader's bounded wait run out. Each bulk-copy
 * wait then expects extra_bytes more than its copies deliver (all copies
 * land, none is left in flight, the barrier phase never completes) and polls
 * at most wait_limit times (wait_limit <= 0: the library's limit). The step
 * kernel then sets ERR_TIMEOUT in the plan status and leaves its work loop.
 * extra_bytes = 0 and wait_limit = 0 restore normal operation. Affects the
 * forward kernels (batched step, single-instance step and operator). */
int shk_check_force_timeout(uint32_t extra_bytes, int64_t wait_limit);

#ifdef __cplusplus
}
#endif

#endif /* SHOCKS_CHECK_H */
