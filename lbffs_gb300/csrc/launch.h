// Host-side launcher declarations shared by the C-ABI layer and the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "lbffs_common.cuh"

namespace lbffs {

struct StepConfig {
    int storage, collision, sgs, wall;
    bool les;  // Smagorinsky with a non-zero LES switch
};

// One half of a time step: bulk=true launches k_bulk, bulk=false launches k_special.
cudaError_t launch_q19(const StepArgs& a, const StepConfig& c, bool bulk, cudaStream_t st);
// row-staged D3Q19 bulk kernel (bulk_tma.cu, one object per storage format)
cudaError_t launch_bulk_tma_s0(const StepArgs& a, int sgs, bool les, cudaStream_t st);
cudaError_t launch_bulk_tma_s1(const StepArgs& a, int sgs, bool les, cudaStream_t st);
cudaError_t launch_bulk_tma_s2(const StepArgs& a, int sgs, bool les, cudaStream_t st);
cudaError_t launch_q27(const StepArgs& a, const StepConfig& c, bool bulk, cudaStream_t st);

// setup.cu
cudaError_t setup_pack_bc(const int* boundary, const int* b1, const int* b2, const int* b3, uint16_t* bc, int nx,
                          int ny, int nz, cudaStream_t st);
cudaError_t setup_classify(int Q, const uint16_t* bc, const uint8_t* solid, const uint8_t* nei, const float* sdf,
                           const float* omega, float omega0, float cs, int damping, uint8_t* flags, uint8_t* scratch,
                           int nx, int ny, int nz, cudaStream_t st);
// compaction of the fluid cells whose flags intersect mask (FL_SPECIAL: the boundary-kernel list):
// counts[nblocks] per chunk of SETUP_CHUNK cells, then scatter
constexpr int SETUP_CHUNK = 256;
cudaError_t setup_count_special(const uint8_t* flags, long long E, uint8_t mask, unsigned* counts, cudaStream_t st);
cudaError_t setup_scatter_special(const uint8_t* flags, long long E, uint8_t mask, const unsigned long long* offsets,
                                  uint32_t* out, cudaStream_t st);
cudaError_t setup_link_masks(int Q, const uint32_t* special, long long n, const uint16_t* bc, const uint8_t* solid,
                             const uint8_t* nei, int nx, int ny, int nz, uint32_t* masks, cudaStream_t st);
// rows [row0, row0 + nrows) of the packed population array (Q*ny*nz rows of nx floats) to / from
// the padded device planes (encode: into dst, and into dst2 when it is set); the packed array may be
// pinned host memory the device addresses directly
cudaError_t encode_f(int storage, int Q, const float* src, void* dst, void* dst2, long long row0, long long nrows,
                     const PadGeom& g, cudaStream_t st);
cudaError_t decode_f(int storage, int Q, const void* src, float* dst, long long row0, long long nrows,
                     const PadGeom& g, cudaStream_t st);
// ghost layer of the population planes f (element size tsize): the face streaming of the six faces
cudaError_t halo_fill(int Q, int tsize, void* f, const uint8_t* flags, const uint16_t* bc, const PadGeom& g,
                      cudaStream_t st);
cudaError_t fill_f32(float* p, float v, long long n, cudaStream_t st);
// out[0] bit 0: a WallFunction code present, bit 1: an invalid code present (out[1]: the largest)
cudaError_t setup_check_codes(const int* b1, const int* b2, const int* b3, long long E, int* out, cudaStream_t st);
// *bad |= 1 unless every face carries one boundary code per axis (codes: code of axis d on the low /
// high face s in bits 3 (2 d + s)) and the face flag (boundary) is set on exactly the border cells:
// the condition under which the step kernels can pull across the border without a ghost layer
cudaError_t setup_check_faces(const int* boundary, const int* b1, const int* b2, const int* b3, int codes, int nx,
                              int ny, int nz, int* bad, cudaStream_t st);
// counts[4] (zeroed by the caller): fluid, special, STL-link and macroscopic-storing cells
cudaError_t setup_count_flags(const uint8_t* flags, long long E, unsigned long long* counts, cudaStream_t st);
// FP64 partial sums: force over the listed cells (3 per block), mass over fluid cells (1 per block)
constexpr int REDUCE_BS = 256;
cudaError_t reduce_force(const uint32_t* cells, long long n, const float* fx, const float* fy, const float* fz,
                         double* partial, int nblocks, cudaStream_t st);
cudaError_t reduce_mass(int storage, int Q, const void* f, const uint8_t* flags, long long E, const PadGeom& g,
                        double* partial, int nblocks, cudaStream_t st);

// lbffs_api.cu: record the message lbffs_last_error(NULL) returns on this thread
void set_thread_error(const std::string& msg);

}  // namespace lbffs
