// Instantiates the reference CPU gridder with its nearest-neighbour convolution policy on the
// sampling function.  TEST INFRASTRUCTURE ONLY: compiled by oracle/build_ref.sh against the
// reference's headers where they lie, into oracle/_ref/; it pins the integer sampling counts of
// the oracle (oracle/bullseye_oracle.c, oracle_sampling_counts_nn) and of the GPU library.
//
// The reference ships convolution_policy<..., convolution_NN> (cpu_algorithm/convolution_policies.h:35-65)
// but no entry point that uses it; this file composes it the way wrapper.cpp:383-425 composes
// grid_sampling_function / facet_sampling_function with the AA and w-projection policies.
#include <cstddef>

#include "templated_gridder.h"

extern "C" void ref_sampling_counts_nn(gridding_parameters *params, int faceting) {
  typedef imaging::correlation_gridding_policy<imaging::grid_sampling_function> corr;
  typedef imaging::phase_transform_policy<imaging::disable_faceting_phase_shift> phase;
  typedef imaging::convolution_policy<corr, imaging::convolution_NN> conv;
  if (faceting) {
    typedef imaging::baseline_transform_policy<imaging::transform_planar_approx_with_w> xform;
    imaging::templated_gridder<corr, xform, phase, conv>(*params);
  } else {
    typedef imaging::baseline_transform_policy<imaging::transform_disable_facet_rotation> xform;
    imaging::templated_gridder<corr, xform, phase, conv>(*params);
  }
}
