// ns_check.cuh -- index checks of the checked build (-DNS_CHECKED).
//
// The checked build of libns_gb300.so range-checks the indices each kernel
// derives before it uses them: shared-tile rows and columns, halo and
// closure offsets, the segment walks of the filter sweeps and the work-list
// items of the batched sweep.  A failed check records where it failed in the
// kernel's error word (a code carrying the file and line, the first failure
// wins) and returns from the enclosing function without the access; it never
// traps, so the context stays usable and the host reports NS_ERR_CHECK.  In
// the ordinary build every check compiles to nothing.
#pragma once

namespace ns {

// Error-word values: 1 is a bounded wait that gave up; a failed index check
// stores kCheckTag | file << 16 | line.
constexpr int kCheckTag = 1 << 24;
enum CheckFile {
    kChkKernels = 1,  // ns_kernels.cu
    kChkSplit = 2,    // ns_split.cu
    kChkBatch = 3,    // ns_batch.cu
    kChkAdjoint = 4,  // ns_adjoint.cu
};

__device__ __forceinline__ void check_fail(int *err, int file, int line)
{
    if (err) atomicCAS(err, 0, kCheckTag | (file << 16) | line);
}

}  // namespace ns

#ifdef NS_CHECKED
#define NS_CHECK(err, file, cond)                      \
    do {                                               \
        if (!(cond)) {                                 \
            ::ns::check_fail((err), (file), __LINE__); \
            return;                                    \
        }                                              \
    } while (0)
// The same for a function that returns a value: returns `ret`.
#define NS_CHECK_RET(err, file, cond, ret)             \
    do {                                               \
        if (!(cond)) {                                 \
            ::ns::check_fail((err), (file), __LINE__); \
            return ret;                                \
        }                                              \
    } while (0)
#else
#define NS_CHECK(err, file, cond) \
    do {                          \
    } while (0)
#define NS_CHECK_RET(err, file, cond, ret) \
    do {                                   \
    } while (0)
#endif
