/*
 * Single-process stand-in for the MPI C interface.
 *
 * Test infrastructure only: it lets the reference library's own CPU sources
 * (which include <mpi.h> from every translation unit) compile and run as one
 * rank, so the reference CPU provider can serve as the parity oracle for the
 * lattice hot path.  World size is 1 and rank is 0; collectives copy the send
 * buffer to the receive buffer (the single-rank result of any reduction); the
 * point-to-point and one-sided calls are only reached by the multi-rank tree
 * modes and fail with MPI_ERR_OTHER if they are ever called.
 *
 * Nothing in the GPU product links against this header.
 */
#ifndef ORACLE_MPI_STUB_H
#define ORACLE_MPI_STUB_H

#include <stddef.h>
#include <stdint.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Win;
typedef int MPI_Info;
typedef ptrdiff_t MPI_Aint;
typedef struct {
	int MPI_SOURCE;
	int MPI_TAG;
	int MPI_ERROR;
} MPI_Status;
typedef void MPI_User_function(void *invec, void *inoutvec, int *len, MPI_Datatype *datatype);

#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_MAX_ERROR_STRING 256
#define MPI_COMM_WORLD 1
#define MPI_INFO_NULL 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

/* Built-in datatypes: the handle is an index into oracle_mpi_type_size(). */
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_FLOAT 3
#define MPI_UINT8_T 4
#define MPI_UINT16_T 5
#define MPI_UINT32_T 6
#define MPI_UINT64_T 7
#define ORACLE_MPI_FIRST_DERIVED 16
#define ORACLE_MPI_MAX_DERIVED 64

#define MPI_SUM 1
#define MPI_MAX 2
#define ORACLE_MPI_FIRST_USER_OP 16

/* Extents of derived (struct) datatypes, filled by MPI_Type_create_struct. */
static inline MPI_Aint *oracle_mpi_derived_extent(void)
{
	static MPI_Aint extents[ORACLE_MPI_MAX_DERIVED];
	return extents;
}

static inline int *oracle_mpi_derived_count(void)
{
	static int count = 0;
	return &count;
}

static inline MPI_Aint oracle_mpi_type_size(MPI_Datatype type)
{
	switch (type)
	{
	case MPI_INT:
		return (MPI_Aint)sizeof(int);
	case MPI_DOUBLE:
		return 8;
	case MPI_FLOAT:
		return 4;
	case MPI_UINT8_T:
		return 1;
	case MPI_UINT16_T:
		return 2;
	case MPI_UINT32_T:
		return 4;
	case MPI_UINT64_T:
		return 8;
	default:
		break;
	}
	if (type >= ORACLE_MPI_FIRST_DERIVED && type < ORACLE_MPI_FIRST_DERIVED + ORACLE_MPI_MAX_DERIVED)
		return oracle_mpi_derived_extent()[type - ORACLE_MPI_FIRST_DERIVED];
	return 0;
}

static inline int oracle_mpi_copy(const void *send, void *recv, int count, MPI_Datatype type)
{
	if (send == MPI_IN_PLACE || send == recv || count <= 0)
		return MPI_SUCCESS;
	const MPI_Aint bytes = oracle_mpi_type_size(type) * (MPI_Aint)count;
	if (bytes <= 0)
		return MPI_ERR_OTHER;
	memmove(recv, send, (size_t)bytes);
	return MPI_SUCCESS;
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Initialized(int *flag) { *flag = 1; return MPI_SUCCESS; }
static inline int MPI_Abort(MPI_Comm comm, int code) { (void)comm; (void)code; return MPI_ERR_OTHER; }
static inline int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }

static inline int MPI_Error_string(int code, char *text, int *length)
{
	const char *message = code == MPI_SUCCESS ? "success" : "single-rank stub: call not supported";
	strcpy(text, message);
	*length = (int)strlen(message);
	return MPI_SUCCESS;
}

static inline int MPI_Get_address(const void *location, MPI_Aint *address)
{
	*address = (MPI_Aint)(uintptr_t)location;
	return MPI_SUCCESS;
}

static inline MPI_Aint MPI_Aint_diff(MPI_Aint a, MPI_Aint b) { return a - b; }

static inline int MPI_Type_create_struct(int count, const int lengths[], const MPI_Aint displacements[],
										 const MPI_Datatype types[], MPI_Datatype *newtype)
{
	int *used = oracle_mpi_derived_count();
	if (*used >= ORACLE_MPI_MAX_DERIVED)
		return MPI_ERR_OTHER;
	MPI_Aint extent = 0;
	for (int i = 0; i < count; i++)
	{
		const MPI_Aint end = displacements[i] + oracle_mpi_type_size(types[i]) * (MPI_Aint)lengths[i];
		if (end > extent)
			extent = end;
	}
	/* Round the extent up to 8-byte alignment, the padding a C struct of doubles gets. */
	extent = (extent + 7) & ~(MPI_Aint)7;
	oracle_mpi_derived_extent()[*used] = extent;
	*newtype = ORACLE_MPI_FIRST_DERIVED + *used;
	(*used)++;
	return MPI_SUCCESS;
}

static inline int MPI_Type_commit(MPI_Datatype *type) { (void)type; return MPI_SUCCESS; }
static inline int MPI_Type_free(MPI_Datatype *type) { (void)type; return MPI_SUCCESS; }

static inline int MPI_Op_create(MPI_User_function *function, int commute, MPI_Op *op)
{
	(void)function;
	(void)commute;
	*op = ORACLE_MPI_FIRST_USER_OP;
	return MPI_SUCCESS;
}

static inline int MPI_Op_free(MPI_Op *op) { (void)op; return MPI_SUCCESS; }

static inline int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm)
{
	(void)op;
	(void)root;
	(void)comm;
	return oracle_mpi_copy(send, recv, count, type);
}

static inline int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm)
{
	(void)op;
	(void)comm;
	return oracle_mpi_copy(send, recv, count, type);
}

static inline int MPI_Bcast(void *buffer, int count, MPI_Datatype type, int root, MPI_Comm comm)
{
	(void)buffer;
	(void)count;
	(void)type;
	(void)root;
	(void)comm;
	return MPI_SUCCESS;
}

static inline int MPI_Gatherv(const void *send, int send_count, MPI_Datatype send_type, void *recv,
							  const int recv_counts[], const int displacements[], MPI_Datatype recv_type,
							  int root, MPI_Comm comm)
{
	(void)recv_counts;
	(void)recv_type;
	(void)root;
	(void)comm;
	if (send == MPI_IN_PLACE)
		return MPI_SUCCESS;
	return oracle_mpi_copy(send, (char *)recv + (MPI_Aint)displacements[0] * oracle_mpi_type_size(recv_type),
						   send_count, send_type);
}

static inline int MPI_Send(const void *buffer, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm)
{
	(void)buffer; (void)count; (void)type; (void)dest; (void)tag; (void)comm;
	return MPI_ERR_OTHER;
}

static inline int MPI_Recv(void *buffer, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Status *status)
{
	(void)buffer; (void)count; (void)type; (void)source; (void)tag; (void)comm; (void)status;
	return MPI_ERR_OTHER;
}

static inline int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status *status)
{
	(void)source; (void)tag; (void)comm; (void)status;
	return MPI_ERR_OTHER;
}

static inline int MPI_Win_create(void *base, MPI_Aint size, int disp_unit, MPI_Info info, MPI_Comm comm, MPI_Win *win)
{
	(void)base; (void)size; (void)disp_unit; (void)info; (void)comm;
	*win = 1;
	return MPI_SUCCESS;
}

static inline int MPI_Win_fence(int assertion, MPI_Win win) { (void)assertion; (void)win; return MPI_SUCCESS; }
static inline int MPI_Win_free(MPI_Win *win) { (void)win; return MPI_SUCCESS; }

static inline int MPI_Put(const void *origin, int origin_count, MPI_Datatype origin_type, int target_rank,
						  MPI_Aint target_disp, int target_count, MPI_Datatype target_type, MPI_Win win)
{
	(void)origin; (void)origin_count; (void)origin_type; (void)target_rank;
	(void)target_disp; (void)target_count; (void)target_type; (void)win;
	return MPI_ERR_OTHER;
}

#ifdef __cplusplus
}
#endif

#endif
