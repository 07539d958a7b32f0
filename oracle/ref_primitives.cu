// Build unit for the reference's own CUDA kernels
// (quantumsim/pauli_vectors/primitives.cu, GPL, never copied here): the file
// is included from the reference source tree at build time, unchanged, with C
// linkage as PyCUDA's SourceModule compiles it, for sm_103a.  The result,
// oracle/_ref/primitives_sm103a.cubin, is test and reference-arm
// infrastructure only: the parity tests use the reference kernel as a second
// oracle and bench.py's reference arm times it; the product never loads it.
extern "C" {
#include QSGB_REF_PRIMITIVES
}
