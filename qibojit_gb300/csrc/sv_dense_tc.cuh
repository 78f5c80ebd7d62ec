// sv_dense_tc.cuh -- dense k-target gates on the tensor cores (sv_dense_tc.cu).
#pragma once

#include "sv_common.cuh"

namespace sv {

// complex64 states with 4..6 targets run on the tensor cores
bool dense_tc_eligible(int dtype, int k);
// Applies the 2^k x 2^k complex64 `gate` (host, row-major, target[0] the most
// significant bit of the row index) to every index group selected by `q` (sorted bit
// positions of controls and targets), on the context's stream.
int dense_tc_apply(Context* ctx, void* state, int nqubits, const void* gate, const int32_t* targets, int k,
                   const BitList& q);

}  // namespace sv
