/* Pre-include for compiling the reference GQF host path for the tests.
 *
 * TEST INFRASTRUCTURE ONLY: nothing in the product links this.
 *
 * The reference's host bitselect (src/gqf.cu:496-512) uses x86 pdep/tzcnt
 * only when __SSE4_2_ is defined; otherwise it falls through to _select64,
 * whose host branch calls abort() (src/gqf.cu:484-488).  Defining the macro
 * for the host pass only keeps the device pass (which cannot assemble x86
 * asm) untouched.  This makes that build x86-only by construction.
 */
#ifndef __CUDA_ARCH__
#define __SSE4_2_
#endif
