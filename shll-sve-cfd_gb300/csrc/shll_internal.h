// Internal declarations shared by the CUDA translation units of libshll_gb300.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

// device error flags (bitwise OR into one int per context)
#define SHLL_FLAG_NONPOSITIVE 1   // density or temperature <= 0 (or NaN) seen
#define SHLL_FLAG_TIMEOUT 2       // a bounded device-side wait gave up
#define SHLL_FLAG_BADARG 4        // a kernel rejected its launch arguments

struct shll_params;
// the parameter checks of shll_create (SHLL_OK, or SHLL_ERR_ARG with a message in err)
int shll_validate_params(const shll_params* p, char* err, size_t len);

// the reference program's globals, when the loading program defines them (refglobals.cu)
bool shll_ref_program_params(shll_params* p);
void shll_ref_set_step(double dt, double dtdx, double dtdy);

// kernel launches issued by the library (shll_kernel_launches)
void shll_count_launches(long n);

enum { STAGE_U_FROM_P = 0, STAGE_P_FROM_U = 1, STAGE_F_FROM_P = 2, STAGE_UPDATE = 3 };

// Arguments of the plain (reference-arithmetic) kernels.  The constants are the reference's
// REAL-typed values widened to double (exact), converted back inside the launchers.
struct PlainArgs {
    int dim, order, limiter, real_bits;
    int nx, ny;
    const void* Uin;
    void* Uout;   // also the in-place U of the staged kernels
    void* P;      // nv primitive planes followed by the sound-speed plane
    void* fp; void* fm; void* hp; void* hm;
    double R, GAMMA, CV, DT_ON_DX, DT_ON_DY, mc_alpha;
    int* flag;
    cudaStream_t stream;
};

namespace plain_fast {
cudaError_t step(const PlainArgs& a);
cudaError_t stage(const PlainArgs& a, int which);
}
namespace plain_exact {
cudaError_t step(const PlainArgs& a);
cudaError_t stage(const PlainArgs& a, int which);
}
