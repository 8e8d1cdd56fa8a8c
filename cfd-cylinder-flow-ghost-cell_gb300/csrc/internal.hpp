// Interface between the ghost-cell translation unit (ghostmac.cu) and the cut-cell one
// (cutcell.cu): a pressure-only handle built over a cut-cell geometry runs the boundary-
// corrected separable inverse of the ghost path (rectangle transforms, column solves, Schur
// band chain, residual checks and refinement sweeps) on the cut-cell Poisson operator.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <string>

#include "../../include/ghostmac.h"
#include "geometry.hpp"
#include "kernels.cuh"

struct gm_handle;

// the per-thread message of a failed call made without a handle (gm_last_error(NULL))
void gm_internal_set_error(const char* msg);

namespace gmi {

// Pressure-only handle over `g` (filled by gm::build_cutcell_geometry); GM_OK or an error
// class with the message in err.  FP64 operator and inverse; three residual checks per solve.
int pressure_create(gm::Geometry&& g, gm_handle** out, std::string& err);
void pressure_destroy(gm_handle* h);
const gm::Geometry& geometry(const gm_handle* h);
cudaStream_t stream(gm_handle* h);
// streams that capture the bodies of conditional graph nodes (two nesting levels)
cudaStream_t body_stream(gm_handle* h, int level);
// while set, pressure_solve records its refinement sweeps as a WHILE node of the graph being
// captured on stream(h)
void set_capturing(gm_handle* h, bool on);
// Monitored solve of A x = b (full pressure grids on the device, inactive cells ignored in b
// and zero in x) in control slot `slot` (gmk::S_P0..S_P2), then its pressure gate.
void pressure_solve(gm_handle* h, const double* b, double* x, int slot);
// b - A x after the last solve's final check (pressure grid)
const double* pressure_residual(gm_handle* h);
gmk::StepCtl* control(gm_handle* h);
// GM_OK or the class of a failed gate / CUDA error recorded in the control block (message in err)
int check(gm_handle* h, const char* where, std::string& err);
int64_t schur_rank(const gm_handle* h);
// surface point-pressure reconstruction (rows = quadrature points, columns = pressure cells)
struct SurfaceCsr {
  int n;
  const int64_t* ptr;
  const int64_t* col;
  const double* val;
  const double* nwx;
  const double* nwy;
};
SurfaceCsr surface(const gm_handle* h);

}  // namespace gmi

// The legacy step's launches on a stream, without synchronisation (legacy.cu); arrays of the
// state are device memory.
namespace gml {
// doubles of device scratch the calls below need
size_t scratch_doubles(const gm_legacy_state& s);
// u*, v* (predictor_rhs_cpp), ghost velocities, the AB2 step (centred), ghost velocities, and
// the Poisson right-hand side into s.rhs
void predict(const gm_legacy_state& s, double dt, double* scratch, cudaStream_t st);
// the corrector (with the ghost-cell branch's ghost velocities and boundary faces), then
// p = phi (centred) or p += phi
void correct(const gm_legacy_state& s, double dt, double* scratch, cudaStream_t st);
// the step's forces (fx_p, fy_p, fx_v, fy_v) into out[0..3] (device)
void forces(const gm_legacy_state& s, double* scratch, double* out, cudaStream_t st);
}  // namespace gml
