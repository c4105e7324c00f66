/*
 * cbns_host.h — C ABI of the host-side C++ pieces the GPU path keeps on the CPU:
 * the input.txt reader, the mesh and Taylor-Green initial condition, the
 * checkpoint format and the VTK XML writer.  They are rewritten from scratch
 * but keep the reference's formats byte for byte, so files move between the
 * reference and this library.  No CUDA dependency.
 */
#ifndef CBNS_HOST_H
#define CBNS_HOST_H

#include <stdint.h>

#include "cbns_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* read_input (src/read_input.cpp:15-103): 17 whitespace-separated values in the
 * fixed order of cbns_params, then the derived constants (cbns_params_derive).
 * Unlike the reference, a missing file, a short file or an unparsable value is
 * an error (CBNS_ERR_IO / CBNS_ERR_FORMAT) instead of silent garbage. */
cbns_status cbns_host_read_input(const char* path, cbns_params* out);

/* Block3d::gen_mesh (src/Block3d.cpp:208-235): node coordinates x[IM+1], y[JM+1],
 * z[KM+1] of a block whose first cell is (i0, j0, k0) of the global grid. */
cbns_status cbns_host_gen_mesh(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM,
                               uint32_t i0, uint32_t j0, uint32_t k0, double* x, double* y, double* z);

/* Block3d::initial_condition + calc_conservative (src/Block3d.cpp:237-300): the
 * Taylor-Green state in the interior of Q (get_idx_Q layout, ghosts set to 0). */
cbns_status cbns_host_initial_condition(const cbns_params* p, uint32_t IM, uint32_t JM, uint32_t KM,
                                        uint32_t i0, uint32_t j0, uint32_t k0, double* Q);

/* Project-defined (no counterpart in the reference): the Taylor-Green state with
 * a solenoidal velocity perturbation of nmodes random Fourier modes, integer
 * wavevectors 1 <= |k| <= kmax, total amplitude amp, drawn from seed
 * (splitmix64), added to u, v, w before the conversion to conserved variables. */
cbns_status cbns_host_initial_condition_perturbed(const cbns_params* p, uint32_t IM, uint32_t JM,
                                                  uint32_t KM, uint64_t seed, double amp, int nmodes,
                                                  int kmax, double* Q);

/* Block3d::output_bin / read_bin (src/Block3d.cpp:964-987, 318-357): t_cur (f64),
 * IM_G, JM_G, KM_G (u32), then NEQ*IM_G*JM_G*KM_G f64.  read checks the three
 * dimensions (CBNS_ERR_FORMAT on mismatch or truncation). */
cbns_status cbns_host_output_bin(const char* fname, double t_cur, uint32_t IM, uint32_t JM, uint32_t KM,
                                 const double* Q);
cbns_status cbns_host_read_bin(const char* fname, uint32_t IM, uint32_t JM, uint32_t KM, double* Q,
                               double* t_cur);

/* output_vtk_xml (src/output_vtk_xml.cpp:22-48) with Block3d::output_vtr and
 * output_vtm (src/Block3d.cpp:396-500): <dir>/<fname><rank %03d>.vtr (ASCII
 * RectilinearGrid, CellData rho u v w p, "%e ") and, on rank 0, <dir>/<fname>.vtm.
 * Primitive arrays are in the padded get_idx layout.  The text is formatted on
 * every host core (CBNS_HOST_THREADS=n to limit it) and written in order, so the
 * file does not depend on the thread count. */
cbns_status cbns_host_output_vtk_xml(const char* dir, const char* fname, int rank, uint32_t num_blocks,
                                     uint32_t IM, uint32_t JM, uint32_t KM, const double* x,
                                     const double* y, const double* z, const double* rho,
                                     const double* u, const double* v, const double* w,
                                     const double* p);

#ifdef __cplusplus
}
#endif

#endif /* CBNS_HOST_H */
