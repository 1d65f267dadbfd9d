// Compile-only check that the adapter's templates bind to the reference's own
// types: graph_v_of_v<int>, hop_constrained_case_info and
// hop_constrained_two_hop_label, taken from the reference's CPU_HopHL headers
// (compiled with the Boost stand-ins of oracle/shim).
#include <HBPLL/test.h>

#include "hsdl_reference_adapter.hpp"

void adapter_binds_reference(graph_v_of_v<int>& g, hop_constrained_case_info& ci) {
  hsdl_gpu::hop_constrained_two_hop_labels_generation(g, ci);
  hsdl_gpu::hop_constrained_clean_L(ci, 1);
  hsdl_gpu::resident_labels idx(ci.L, ci.upper_k);
  (void)idx.extract_distance(0, 1, ci.upper_k);
  (void)idx.extract_shortest_path(0, 1, ci.upper_k);
}
