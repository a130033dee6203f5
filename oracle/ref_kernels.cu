// ref_kernels.cu -- device code of the reference's own SpMM kernels
// (include/mma_tf32.cuh, found through -I at build time, never copied),
// compiled to a cubin for sm_103a with unmangled names so that a driver-API
// loader can launch them without a host-side build on the GPU machine.
// TEST INFRASTRUCTURE ONLY: the cubin produces the golden SpMM outputs
// (tests/golden/make_ref_spmm.py) that pin the oracle and the product kernels
// to the reference's own results.  Build: make -C oracle refkernels.
#include "mmio.hpp"
#include "ptx_tf32.hpp"

extern "C" {
#include "mma_tf32.cuh"
}
