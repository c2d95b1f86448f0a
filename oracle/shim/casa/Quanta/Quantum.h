/* Empty stand-in for casacore's Quantum.h.  The reference CPU wrapper includes it
 * (bullseye/mo/cpu_algorithm/wrapper.cpp:41) but uses nothing from it.  Test
 * infrastructure only: used when compiling the reference CPU library as the oracle. */
