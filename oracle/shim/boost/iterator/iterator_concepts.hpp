/* Empty stand-in for boost's iterator_concepts.hpp.  The reference includes it
 * (bullseye/mo/cpu_gpu_common/cu_basic_complex.h:40) but uses nothing from it.  Test
 * infrastructure only: used when compiling the reference CPU library as the oracle. */
