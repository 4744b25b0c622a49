/*
 * FFTW-MPI stand-in for compiling the reference with one rank: the slab
 * plan of fftw3d_mpi_create_plan (src/init.c:752-757) becomes the serial
 * FFTW 2.1.5 in-place plan of the same size and direction, and the local
 * slab is the whole grid.
 */
#ifndef MTH_REFSHIM_FFTW_MPI_H
#define MTH_REFSHIM_FFTW_MPI_H
#include <fftw.h>
#include "mpi.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct mth_fftwnd_mpi_plan_s* fftwnd_mpi_plan;
#define FFTW_NORMAL_ORDER 0
#define FFTW_TRANSPOSED_ORDER 1
fftwnd_mpi_plan fftw3d_mpi_create_plan(MPI_Comm c, int nx, int ny, int nz, fftw_direction dir, int flags);
void fftwnd_mpi_local_sizes(fftwnd_mpi_plan p, int* lnx, int* lxs, int* lnyt, int* lyst, int* lsize);
void fftwnd_mpi(fftwnd_mpi_plan p, int n_fields, fftw_complex* data, fftw_complex* work, int order);
void fftwnd_mpi_destroy_plan(fftwnd_mpi_plan p);
#ifdef __cplusplus
}
#endif
#endif
