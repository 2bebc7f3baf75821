// propmr.cuh -- host entry points of the mixed-radix passes (propmr.cu),
// called by the propagation dispatch in prop.cu for lengths that are not
// powers of two.
#pragma once
#include "propdev.cuh"

namespace olg {

// radices for N = 2^a 3^b 5^c (false otherwise)
bool mr_plan(int N, MrPlan *pl);
// a plan exists and one CTA can hold a sequence of length N
bool mr_length_ok(int N);
// fill P's plans, twiddle tables and tile sizes for its non-power-of-two axes
int mr_prepare(PropParams &P);
int mr_rows_pass(const PropParams &P, bool inverse, cudaStream_t st);
int mr_cols_pass(const PropParams &P, cudaStream_t st);
int mr_chirp_axis(const ChirpAxis &A, cudaStream_t st);

} // namespace olg
