// fused.h -- the fused FP64 timestep (fused.cu) and helpers shared by the
// C ABI in interface.cu.
#pragma once

#include "../../include/flow_mesh.h"
#include "stages.h"

namespace flow {

int record_error(int code, const char* fmt, ...);
int check_launch(const char* where);
int check_mesh(const Mesh* m, int nx, int ny, const char* where);
int check_sizes(int nx, int ny, int pad, const char* where);
cudaStream_t current_stream();
int verbose();

// SMs of the current device (cached per device).
int num_sms();
// Calls that may have written the state arrays between two fused steps: every
// entry point taking a mesh (check_mesh) and the other writers count one
// (note_state_write).  A fused step reuses the previous step's tile marks only
// when exactly one such call -- its own -- came between them.
unsigned long long mesh_calls();
void note_state_write();
// Conservation totals of the interior (reduce_array[3..4]) by tiles whose
// partial sums stay in reduce_array's flag region, kept across calls for tiles
// at rest through the fused step between them; false (nothing launched) when
// reduce_array is too small for the region.
bool tile_conservation(int nx, int ny, int pad, const double* rho, const double* e,
                       double* ra, cudaStream_t s);
// Kernel launches issued by this library (the fused step's kernels and the
// conservation totals), for gb300_launch_count.
void count_launches(unsigned n);

// One full timestep with the fused kernels; dt/dt_h stay on the device inside
// the step and are copied to mesh->dt/dt_h before returning.
// one_kernel_lagrangian: the Lagrangian phase as one kernel (lag_fused.cuh)
// instead of the four kernels the mixed and batched steps share.
int fused_solve(Mesh* mesh, int tt, double* P, double* rho, double* rho_old,
                double* e, double* u, double* v, double* rho_u, double* rho_v,
                double* Qxx, double* Qyy, double* F_x, double* F_y,
                double* uF_x, double* uF_y, double* vF_x, double* vF_y,
                double* reduce_array, bool one_kernel_lagrangian);
// Output rows per CTA of the one-kernel Lagrangian phase (1 .. 64).
int set_lagrangian_rows(int rows);

// Mixed form: FP32 bulk arithmetic, FP64 density/energy and their
// conservative updates.  The workspace holds every intermediate array.
size_t mixed_workspace_bytes(int nx, int ny);
// Byte offset of a cell-sized FP64 block of the workspace that is zero after
// mixed_prepare (the first-sweep density, written only during a step).
size_t mixed_zero_block_offset(int nx, int ny);
// Byte offset of the FP32 velocity u (GB300_MIXED_U) or v (GB300_MIXED_V).
size_t mixed_workspace_offset(int nx, int ny, int field);
int mixed_prepare(Mesh* mesh, double* rho, double* e, void* work, size_t bytes);
int mixed_solve(Mesh* mesh, int tt, double* rho, double* e, float* rho_u,
                float* rho_v, void* work, size_t bytes, double* reduce_array);

}  // namespace flow
