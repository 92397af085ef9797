/*
 * cfcull_testing.h — test hooks of libcfcull (no counterpart in the
 * reference, whose VK_CHECK logs an error and carries on:
 * HelloVulkan/Header/Vulkan/VulkanCheck.h:17-19).
 *
 * They let a test drive the library's failure paths without faulting, trapping
 * or hanging a GPU: every wait inside a kernel is bounded, and a run-out wait
 * sets a bit in the context's (or workspace's) device error word, which
 * cf_context_check_device_error reports as CF_ERROR_DEVICE_TIMEOUT; every
 * device allocation failure returns CF_ERROR_OUT_OF_MEMORY.  Not for use in
 * production: the knobs are process-wide.
 */
#ifndef CFCULL_TESTING_H
#define CFCULL_TESTING_H

#include "cfcull.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Stall injections (cf_testing_inject_stall). */
#define CF_TESTING_STALL_ONE_LAUNCH 1u  /* the one-launch kernel's CTA 0 withholds its hit total */
#define CF_TESTING_STALL_BRUTE_FORCE 2u /* the brute-force kernel's CTA 0 never sends its first light tile */

/* Sets the time limit of every bounded wait inside the culling kernels on
 * the current device (0 restores the default of 2 s). */
CFCULL_API int cf_testing_set_wait_limit_ns(uint64_t limit_ns);
/* Makes later culling launches on the current device withhold one part
 * (CF_TESTING_STALL_* bits; 0 turns it off), so that the other threads'
 * bounded waits run out and the kernels report CF_ERROR_DEVICE_TIMEOUT through
 * the device error word.  Nothing is left waiting or in flight: the kernels
 * return after the limit and the context stays usable. */
CFCULL_API int cf_testing_inject_stall(uint32_t mode);
/* Lets the library's next n device allocations through and makes the one
 * after them fail as if the device were out of memory (n = 0: the very next
 * one); n < 0 turns this off.  Covers contexts, the pipelines' buffers and
 * workspaces, batches and servers. */
CFCULL_API int cf_testing_fail_allocation_after(int32_t n);
/* Makes the servers' next n launches of queued light-set uploads and jitters
 * fail as a failed launch would (CF_ERROR_CUDA), without launching anything;
 * n <= 0 turns this off.  The versions they would have written are marked
 * failed, and every request bound to one completes with CF_ERROR_CUDA. */
CFCULL_API int cf_testing_fail_version_writes(int32_t n);

#ifdef __cplusplus
}
#endif

#endif /* CFCULL_TESTING_H */
