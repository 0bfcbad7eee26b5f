/*
 * Single-rank stand-in for the FFTW 2.1.5 MPI interface that SRX calls.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref build). FFTW is not vendored with the
 * reference and is absent here; the transform behind this header is the
 * project's own CPU mixed-radix DFT (oracle/fft_cpu.c), checked against
 * numpy.fft.fftn. Semantics kept from FFTW 2's published interface:
 * 3-D complex-to-complex, in place, unnormalised, exponent sign -1 for
 * FFTW_FORWARD and +1 for FFTW_BACKWARD, row-major [x][y][z] with z fastest,
 * FFTW_NORMAL_ORDER output. Call sites: init.c:753-766, evolution.c:1163,1195,
 * 1411,1424.
 *
 * fftw_malloc pads and zero-fills its allocation: evolution.c:1421 writes one
 * element past the end of fft_data using stale loop indices
 * (px=lnx, py=CellDim[1], pz=CellDim[2]).
 */
#ifndef SRX_SHIM_FFTW_MPI_H
#define SRX_SHIM_FFTW_MPI_H
#include <stddef.h>
#include <mpi.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double re, im; } fftw_complex;
typedef enum { FFTW_FORWARD = -1, FFTW_BACKWARD = 1 } fftw_direction;
typedef enum { FFTW_NORMAL_ORDER = 0, FFTW_TRANSPOSED_ORDER = 1 } fftwnd_mpi_output_order;
#define FFTW_ESTIMATE 0

typedef struct srx_fftwnd_plan *fftwnd_mpi_plan;

fftwnd_mpi_plan fftw3d_mpi_create_plan(MPI_Comm comm, int nx, int ny, int nz,
                                       fftw_direction dir, int flags);
void fftwnd_mpi_local_sizes(fftwnd_mpi_plan p, int *local_nx, int *local_x_start,
                            int *local_ny_after_transpose,
                            int *local_y_start_after_transpose, int *total_local_size);
void fftwnd_mpi(fftwnd_mpi_plan p, int n_fields, fftw_complex *local_data,
                fftw_complex *work, fftwnd_mpi_output_order order);
void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
