// vibe-model_gb300/csrc/tlad_internal.cuh
//
// Device-side access to a vibe_tlad object for runs that linearise about a
// trajectory held on the device (the model's state buffers share the TL/AD
// device layout: element (i,j,k) at (k*(ny+1)+j)*P+i, P = nx+1 rounded up to 8).
#pragma once
#include <cuda_runtime.h>

struct vibe_tlad;

namespace vgb {
void tlad_grid(const vibe_tlad* t, int* nx, int* ny, int* nz);
cudaStream_t tlad_stream(vibe_tlad* t);
double* const* tlad_work(vibe_tlad* t, int s);  // work states 0..3 are free for the caller
// linearisation point of the next TL/AD steps (12 device fields); nullptr = the set base
void tlad_use_base(vibe_tlad* t, double* const* base);
void tlad_tl_step(vibe_tlad* t, double* const* in, double* const* out, double dt);   // uses work 4
void tlad_ad_step(vibe_tlad* t, double* const* bo, double* const* bi, double dt);   // uses work 4, 5
bool tlad_upload(vibe_tlad* t, const double* const* host, double* const* dst);
bool tlad_download(vibe_tlad* t, double* const* src, const double* const* keep, double* const* host);
void tlad_set_error(const char* msg);
}  // namespace vgb
