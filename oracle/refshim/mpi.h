/*
 * Stand-in for the subset of MPI that the reference's src/ uses (test
 * infrastructure, not MPI).  The ranks of a run are threads of one process
 * (ref_harness.cpp starts them); each thread knows its rank.  Point-to-point
 * messages are buffered at the send and matched by (source, destination,
 * tag); collectives meet at a barrier and combine the ranks' values in rank
 * order; MPI-IO writes through one shared file descriptor with pwrite at the
 * offsets of the file view (a displacement plus a filetype of repeated
 * subarrays, as src/lbm.cpp:593-609 builds it).
 */
#ifndef IMEXREF_MPI_H
#define IMEXREF_MPI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef struct imexref_type* MPI_Datatype;
typedef int MPI_Op;
typedef struct imexref_request* MPI_Request;
typedef struct imexref_file* MPI_File;
typedef long long MPI_Offset;
typedef int MPI_Info;
typedef struct MPI_Status {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_SUCCESS 0
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_REQUEST_NULL ((MPI_Request)0)
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4
#define MPI_MODE_RDWR 8
#define MPI_SEEK_SET 600
#define MPI_ORDER_C 56
#define MPI_ORDER_FORTRAN 57

extern struct imexref_type imexref_int, imexref_double, imexref_float, imexref_char;
#define MPI_INT (&imexref_int)
#define MPI_DOUBLE (&imexref_double)
#define MPI_REAL (&imexref_float)
#define MPI_FLOAT (&imexref_float)
#define MPI_CHAR (&imexref_char)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses);

int MPI_Type_create_subarray(int ndims, const int* sizes, const int* subsizes, const int* starts, int order,
                             MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);

int MPI_File_open(MPI_Comm comm, const char* name, int amode, MPI_Info info, MPI_File* fh);
int MPI_File_close(MPI_File* fh);
int MPI_File_seek(MPI_File fh, MPI_Offset offset, int whence);
int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype type, MPI_Status* status);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype, const char* datarep,
                      MPI_Info info);
int MPI_File_write_all(MPI_File fh, const void* buf, int count, MPI_Datatype type, MPI_Status* status);

#ifdef __cplusplus
}
#endif
#endif /* IMEXREF_MPI_H */
