// pt_wavefront_checked.cu — the wavefront kernels built a second time with
// index checks (PT_DEBUG_CHECKS), in place of a memory checker for the
// queue code: every queue append, slot read from a queue or the free list,
// pass index and sample index is checked before use; a failed check records
// its site and index in the counters and skips the access, and the host
// turns it into PT_ERR_KERNEL (pt_set_device_checks, pt_batch_set_device_checks).
// Results with the checks passing are the default kernels' bit for bit.
#define PT_DEBUG_CHECKS 1
#define PTK_WF(name) name##_checked
#include "pt_wavefront.cu"
