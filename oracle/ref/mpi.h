// Single-rank stand-in for <mpi.h>, used only to compile the reference C++
// sources into the golden-vector harness (oracle/ref/harness.cpp).
//
// This is test infrastructure: it lets the reference's MPI wrappers
// (src/MPIMethods.h) run as a world of one rank, where a broadcast is a no-op
// and every reduction or gather is a copy of the local buffer.  Datatype
// handles carry their element size in bytes so the copies need no table.
#pragma once

#include <cstddef>
#include <cstring>
#include <iostream>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_LONG_LONG_INT ((MPI_Datatype)sizeof(long long))
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_SUCCESS 0

inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
inline int MPI_Get_processor_name(char* name, int* len)
{
	std::strcpy(name, "stub");
	*len = 4;
	return MPI_SUCCESS;
}
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

inline void mpi_stub_copy(const void* src, void* dst, int count, MPI_Datatype type)
{
	if (src != dst && count > 0)
	{
		std::memmove(dst, src, (size_t)count * (size_t)type);
	}
}

inline int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op, int, MPI_Comm)
{
	mpi_stub_copy(send, recv, count, type);
	return MPI_SUCCESS;
}
inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op, MPI_Comm)
{
	mpi_stub_copy(send, recv, count, type);
	return MPI_SUCCESS;
}
inline int MPI_Gather(const void* send, int scount, MPI_Datatype stype, void* recv, int, MPI_Datatype, int, MPI_Comm)
{
	mpi_stub_copy(send, recv, scount, stype);
	return MPI_SUCCESS;
}
