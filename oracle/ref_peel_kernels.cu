// TEST INFRASTRUCTURE ONLY.  Translation unit that compiles the reference's
// variant-1 peel kernels (selectNodesAtLevel1 and processNodes1,
// src/ours.cc:2-114, with the queue helpers of src/buffer.cc) unmodified into
// a cubin for sm_103a, exactly as main.cu pulls them in (main.cu:6-9).  The
// reference host loop around them is replayed by oracle/ref_peel_driver.cpp.
#include "gpu_memory_allocation.h"
#include "buffer.cc"
#include "ours.cc"
