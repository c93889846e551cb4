/*
 * hostmpi: the CPU oracle and CPU baseline of the device MPI runtime.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this; the
 * tests, the smoke check and the benchmark's CPU-baseline leg run programs
 * built against it to produce reference results on host cores.
 *
 * One process per rank (fork), shared-memory mailboxes, the same C API subset
 * as the device runtime, and the reference's own collective algorithms:
 * flat root fan-out for Bcast/Gather/Scatter, root fold in rank order for
 * Reduce (gpu_libs/gpu_mpi/mpi.cu:200-225 with operators.cu:216-218),
 * Allreduce = Reduce + Bcast (mpi.cu:276-282), Alltoallv as P-1 Isend/Irecv
 * pairs (mpi.cu:363-408), Comm_split by (key, rank) (communicator.cu:154-199).
 * Defects of the reference are not reproduced: status is filled, wildcards
 * match in every order, Sendrecv exchanges data.
 */
#ifndef HOSTMPI_MPI_H
#define HOSTMPI_MPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPI_SUCCESS 0
#define MPI_FAILURE -1
#define MPI_ERR_OTHER 1
#define MPI_ERR_BUFFER 2
#define MPI_ERR_COUNT 3
#define MPI_ERR_TYPE 4
#define MPI_ERR_TAG 5
#define MPI_ERR_COMM 6
#define MPI_ERR_RANK 7
#define MPI_ERR_REQUEST 8
#define MPI_ERR_ROOT 9
#define MPI_ERR_OP 10
#define MPI_ERR_ARG 11
#define MPI_ERR_TRUNCATE 12
#define MPI_ERR_INTERN 13
#define MPI_ERR_NO_MEM 14
#define MPI_UNDEFINED -1
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_MAX_ERROR_STRING 256
#define MPI_ANY_TAG (-1)
#define MPI_ANY_SOURCE (-1)
#define MPI_PROC_NULL (-2)
#define MPI_TAG_UB ((1 << 15) - 1)
#define MPI_THREAD_SINGLE 1
#define MPI_THREAD_FUNNELED 2
#define MPI_THREAD_SERIALIZED 3
#define MPI_THREAD_MULTIPLE 4
#define MPI_IDENT 0
#define MPI_CONGRUENT 1
#define MPI_SIMILAR 2
#define MPI_UNEQUAL 3

/* Same names, same order as the device MPI_Datatype enum. */
typedef enum MPI_Datatype {
    MPI_CHAR, MPI_SHORT, MPI_INT, MPI_LONG, MPI_LONG_LONG_INT, MPI_LONG_LONG, MPI_SIGNED_CHAR,
    MPI_UNSIGNED_CHAR, MPI_UNSIGNED_SHORT, MPI_UNSIGNED, MPI_UNSIGNED_LONG,
    MPI_UNSIGNED_LONG_LONG, MPI_FLOAT, MPI_DOUBLE, MPI_LONG_DOUBLE, MPI_WCHAR, MPI_C_BOOL,
    MPI_INT8_T, MPI_INT16_T, MPI_INT32_T, MPI_INT64_T, MPI_UINT8_T, MPI_UINT16_T,
    MPI_UINT32_T, MPI_UINT64_T, MPI_C_COMPLEX, MPI_C_FLOAT_COMPLEX, MPI_C_DOUBLE_COMPLEX,
    MPI_C_LONG_DOUBLE_COMPLEX, MPI_BYTE, MPI_2INT, MPI_FLOAT_INT, MPI_DOUBLE_INT, MPI_LONG_INT,
    MPI_PACKED,
    HOSTMPI_NUM_BASIC_TYPES,
    MPI_DATATYPE_NULL = 0x7fff,
    HOSTMPI_FIRST_DERIVED_TYPE = 0x8000
} MPI_Datatype;

typedef struct hostmpi_comm* MPI_Comm;
typedef struct hostmpi_group* MPI_Group;
typedef struct hostmpi_op* MPI_Op;
typedef struct hostmpi_request* MPI_Request;

typedef struct MPI_Status {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
    int hostmpi_count_lo;
    int hostmpi_count_hi;
} MPI_Status;

typedef void MPI_User_function(void* invec, void* inoutvec, int* len, MPI_Datatype* datatype);
typedef int MPI_Copy_function(MPI_Comm, int, void*, void*, void*, int*);
typedef int MPI_Delete_function(MPI_Comm, int, void*, void*);

extern MPI_Comm MPI_COMM_WORLD;
extern MPI_Comm MPI_COMM_SELF;
extern MPI_Group MPI_GROUP_WORLD;
extern MPI_Group MPI_GROUP_EMPTY;
extern MPI_Op MPI_MAX, MPI_MIN, MPI_SUM, MPI_PROD, MPI_LAND, MPI_BAND, MPI_LOR, MPI_BOR,
    MPI_LXOR, MPI_BXOR, MPI_MAXLOC, MPI_MINLOC;

#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_GROUP_NULL ((MPI_Group)0)
#define MPI_OP_NULL ((MPI_Op)0)
#define MPI_REQUEST_NULL ((MPI_Request)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_IN_PLACE ((void*)-1)
#define MPI_BOTTOM ((void*)0)

int MPI_Init(int* argc, char*** argv);
int MPI_Init_thread(int* argc, char*** argv, int required, int* provided);
int MPI_Initialized(int* flag);
int MPI_Finalize(void);
int MPI_Finalized(int* flag);
int MPI_Abort(MPI_Comm comm, int errorcode);
int MPI_Get_processor_name(char* name, int* resultlen);
int MPI_Error_string(int errorcode, char* string, int* resultlen);
double MPI_Wtime(void);
double MPI_Wtick(void);
int MPI_Type_size(MPI_Datatype datatype, int* size);
int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* datatype);
int MPI_Type_free(MPI_Datatype* datatype);
int MPI_Get_count(const MPI_Status* status, MPI_Datatype datatype, int* count);

int MPI_Send(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm);
int MPI_Ssend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm,
             MPI_Status* status);
int MPI_Isend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm,
              MPI_Request* request);
int MPI_Irecv(void* buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm,
              MPI_Request* request);
int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status* status);
int MPI_Sendrecv_replace(void* buf, int count, MPI_Datatype datatype, int dest, int sendtag,
                         int source, int recvtag, MPI_Comm comm, MPI_Status* status);
int MPI_Wait(MPI_Request* request, MPI_Status* status);
int MPI_Waitall(int count, MPI_Request array_of_requests[], MPI_Status* array_of_statuses);
int MPI_Waitany(int count, MPI_Request array_of_requests[], int* index, MPI_Status* status);
int MPI_Waitsome(int incount, MPI_Request array_of_requests[], int* outcount,
                 int array_of_indices[], MPI_Status array_of_statuses[]);
int MPI_Test(MPI_Request* request, int* flag, MPI_Status* status);
int MPI_Testall(int count, MPI_Request array_of_requests[], int* flag,
                MPI_Status array_of_statuses[]);
int MPI_Request_free(MPI_Request* request);
int MPI_Iprobe(int source, int tag, MPI_Comm comm, int* flag, MPI_Status* status);
int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status* status);

int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void* buffer, int count, MPI_Datatype datatype, int root, MPI_Comm comm);
int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
               int root, MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
                  MPI_Comm comm);
int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
               int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Gatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                const int recvcounts[], const int displs[], MPI_Datatype recvtype, int root,
                MPI_Comm comm);
int MPI_Scatter(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Scatterv(const void* sendbuf, const int sendcounts[], const int displs[],
                 MPI_Datatype sendtype, void* recvbuf, int recvcount, MPI_Datatype recvtype,
                 int root, MPI_Comm comm);
int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                  int recvcount, MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Allgatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                   const int recvcounts[], const int displs[], MPI_Datatype recvtype,
                   MPI_Comm comm);
int MPI_Alltoall(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                 int recvcount, MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Alltoallv(const void* sendbuf, const int sendcounts[], const int sdispls[],
                  MPI_Datatype sendtype, void* recvbuf, const int recvcounts[],
                  const int rdispls[], MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Reduce_scatter_block(const void* sendbuf, void* recvbuf, int recvcount,
                             MPI_Datatype datatype, MPI_Op op, MPI_Comm comm);
int MPI_Scan(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
             MPI_Comm comm);
int MPI_Exscan(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
               MPI_Comm comm);

int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* newcomm);
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* newcomm);
int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm* newcomm);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Comm_group(MPI_Comm comm, MPI_Group* group);
int MPI_Comm_compare(MPI_Comm comm1, MPI_Comm comm2, int* result);
int MPI_Group_incl(MPI_Group group, int n, const int ranks[], MPI_Group* newgroup);
int MPI_Group_excl(MPI_Group group, int n, const int ranks[], MPI_Group* newgroup);
int MPI_Group_range_incl(MPI_Group group, int n, int ranges[][3], MPI_Group* newgroup);
int MPI_Group_free(MPI_Group* group);
int MPI_Group_size(MPI_Group group, int* size);
int MPI_Group_rank(MPI_Group group, int* rank);
int MPI_Group_translate_ranks(MPI_Group group1, int n, const int ranks1[], MPI_Group group2,
                              int ranks2[]);
int MPI_Cart_create(MPI_Comm comm_old, int ndims, const int dims[], const int periods[],
                    int reorder, MPI_Comm* comm_cart);
int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm* comm_new);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]);
int MPI_Cart_rank(MPI_Comm comm, const int coords[], int* rank);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int* rank_source, int* rank_dest);
int MPI_Dims_create(int nnodes, int ndims, int dims[]);
int MPI_Attr_get(MPI_Comm comm, int keyval, void* attribute_val, int* flag);
int MPI_Attr_put(MPI_Comm comm, int keyval, void* attribute_val);
int MPI_Keyval_create(MPI_Copy_function* copy_fn, MPI_Delete_function* delete_fn, int* keyval,
                      void* extra_state);
int MPI_Op_create(MPI_User_function* user_fn, int commute, MPI_Op* op);
int MPI_Op_free(MPI_Op* op);

#ifdef __cplusplus
}
#endif

#endif
