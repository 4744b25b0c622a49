/*
 * Single-rank MPI stand-in used only to compile the reference M-THEMES
 * sources (for pinning the oracle).  It covers exactly the calls the
 * reference's build makes (MPI_Init ... MPI_File_write); every collective is
 * a copy from the send to the receive buffer, which is what MPI does with
 * one rank.  Point-to-point MPI_Send/MPI_Recv abort: with one rank the
 * reference never reaches them (they sit behind `NumPE>1` or `mpirank>0`).
 */
#ifndef MTH_REFSHIM_MPI_H
#define MTH_REFSHIM_MPI_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef struct mth_mpi_file* MPI_File;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_FLOAT 3
#define MPI_CHAR 4
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_INFO_NULL 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4
#define MPI_SUCCESS 0

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm c, int* n);
int MPI_Comm_rank(MPI_Comm c, int* r);
int MPI_Barrier(MPI_Comm c);
int MPI_Abort(MPI_Comm c, int code);
int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Allgather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, MPI_Comm c);
int MPI_Allgatherv(const void* s, int sc, MPI_Datatype st, void* r, const int* rcounts, const int* displs,
                   MPI_Datatype rt, MPI_Comm c);
int MPI_Send(const void* b, int n, MPI_Datatype t, int dest, int tag, MPI_Comm c);
int MPI_Recv(void* b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status* st);
int MPI_Sendrecv(const void* sb, int sc, MPI_Datatype st, int dest, int stag, void* rb, int rc,
                 MPI_Datatype rt, int src, int rtag, MPI_Comm c, MPI_Status* s);
int MPI_Address(void* p, MPI_Aint* a);
int MPI_Type_struct(int count, int* blocklens, MPI_Aint* disps, MPI_Datatype* types, MPI_Datatype* out);
int MPI_Type_commit(MPI_Datatype* t);
int MPI_Type_extent(MPI_Datatype t, MPI_Aint* e);
int MPI_File_open(MPI_Comm c, const char* name, int amode, MPI_Info info, MPI_File* fh);
int MPI_File_set_view(MPI_File fh, long long disp, MPI_Datatype et, MPI_Datatype ft, const char* rep, MPI_Info info);
int MPI_File_write(MPI_File fh, const void* b, int n, MPI_Datatype t, MPI_Status* st);
int MPI_File_close(MPI_File* fh);
#ifdef __cplusplus
}
#endif
#endif
