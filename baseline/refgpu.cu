// One translation unit holding the reference's device code, so that it can
// be compiled to a stand-alone sm_103a cubin without device linking.  This
// file only includes the reference's sources where they lie (-I to the
// reference tree); it adds nothing to them.
//
// TEST INFRASTRUCTURE ONLY: the reference's own CUDA build, timed beside the
// product by oracle/refgpu.py.
#include "hashutil.cu"
#include "gqf.cu"
