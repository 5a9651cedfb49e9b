// Occupancy query of the reference-arithmetic batch kernel (defined in mmf_exact.cu).
#pragma once
namespace mmf {
int batch_max_blocks_per_sm_exact(int order);
int batch_slope_blocks_per_sm_exact();
}
