// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// Link stubs for building the reference's CPU path from its own sources without a CUDA
// runtime.  The reference's CPU branches (useGPU == false) never call the GPU launchers
// below; GPUArray::allocate/deallocate call cudaMalloc/cudaFree unconditionally and ignore the
// result (inc/gpuarray.h:282-311), so those return "no device" and do nothing.  Any stubbed
// launcher that is reached aborts, which would mean the reference left its CPU path.
#include <cstdio>
#include <cstdlib>
#include "curand_kernel.h"
#include "sphericalVertexModel.cuh"
#include "simpleModel.cuh"
#include "utilities.cuh"
#include "hyperrectangularCellList.cuh"
#include "noiseSource.cuh"
#include "neighborList.cuh"
#include "brownianDynamics.cuh"
#include "energyMinimizerFIRE.cuh"
#include "velocityVerlet.cuh"
#include "vectorialVicsek.cuh"

[[noreturn]] static void offPath(const char* name) {
    std::fprintf(stderr, "reference CPU build: GPU launcher %s reached\n", name);
    std::abort();
}

bool gpu_move_particles_on_sphere(dVec*, dVec*, sphericalDomain&, scalar, int) { offPath(__func__); }
bool gpu_selfPropelledParticleDisplacement(dVec*, dVec*, dVec*, scalar, scalar, scalar, int) { offPath(__func__); }
bool gpu_vectorVicsek_target_directors(dVec*, dVec*, unsigned int*, int*, curandState*, Index2D&, scalar, int) { offPath(__func__); }
bool gpu_vectorVicsek_update_directors(dVec*, dVec*, scalar, scalar, int) { offPath(__func__); }
bool gpu_spherical_vertex_model_geometry(dVec*, dVec*, int*, int*, unsigned int*, dVec*, dVec*, dVec*, unsigned int*, scalar2*, Index2D, Index2D, sphericalDomain&, int) { offPath(__func__); }
bool gpu_quadratic_spherical_cellular_force(dVec*, dVec*, dVec*, int*, unsigned int*, dVec*, dVec*, dVec*, unsigned int*, scalar2*, scalar2*, Index2D, scalar, sphericalDomain&, int) { offPath(__func__); }
bool gpu_vm_test_edges_for_T1(dVec*, int*, int*, int*, unsigned int*, int*, sphericalDomain&, scalar, int, int, int*, Index2D&) { offPath(__func__); }
bool gpu_vm_parse_multiple_flips(int*, int*, int*, int*, unsigned int*, int*, int*, int*, int4*, Index2D&, int) { offPath(__func__); }
bool gpu_vm_flip_edges(int*, dVec*, int*, int*, unsigned int*, int*, int*, int4*, sphericalDomain&, Index2D&, int, int) { offPath(__func__); }
bool gpu_move_particles(dVec*, dVec*, periodicBoundaryConditions&, scalar, int) { offPath(__func__); }
bool gpu_zero_array(scalar*, int) { offPath(__func__); }
bool gpu_zero_array(int*, int) { offPath(__func__); }
bool gpu_zero_array(unsigned int*, int) { offPath(__func__); }
bool gpu_zero_array(dVec*, int) { offPath(__func__); }
bool gpu_dVec_dot_products(dVec*, dVec*, scalar*, scalar*, int, int, int) { offPath(__func__); }
bool gpu_compute_cell_list(dVec*, unsigned int*, int*, dVec*, int, int&, iVec, dVec, scalar, IndexDD&, Index2D&, int*) { offPath(__func__); }
bool gpu_initialize_RNG_array(curandState*, int, int, int) { offPath(__func__); }
bool gpu_compute_neighbor_list(int*, unsigned int*, dVec*, unsigned int*, int*, dVec*, dVec*, int*, int*, periodicBoundaryConditions&, scalar, Index2D, Index2D, IndexDD, Index2D, int, iVec, dVec, int, scalar, int, int, int, bool) { offPath(__func__); }
bool gpu_brownian_eom_integration(dVec*, dVec*, curandState*, int, scalar, scalar, scalar) { offPath(__func__); }
bool gpu_update_velocity_FIRE(dVec*, dVec*, scalar, scalar, int) { offPath(__func__); }
bool gpu_update_velocity(dVec*, dVec*, scalar*, scalar, int) { offPath(__func__); }
bool gpu_displacement_velocity_verlet(dVec*, dVec*, dVec*, scalar*, scalar, int) { offPath(__func__); }

extern "C" {
cudaError_t cudaMalloc(void** p, size_t) { if (p) *p = nullptr; return cudaErrorNoDevice; }
cudaError_t cudaFree(void*) { return cudaSuccess; }
cudaError_t cudaMemcpy(void*, const void*, size_t, cudaMemcpyKind) { return cudaErrorNoDevice; }
cudaError_t cudaMemset(void*, int, size_t) { return cudaErrorNoDevice; }
cudaError_t cudaEventCreate(cudaEvent_t* e) { if (e) *e = nullptr; return cudaErrorNoDevice; }
cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaErrorNoDevice; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaErrorNoDevice; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) { if (ms) *ms = 0.f; return cudaErrorNoDevice; }
}
