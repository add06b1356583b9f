/*
 * Single-rank stand-in for the MPI API surface that meso-lts calls.
 *
 * Test infrastructure only: it lets the unmodified meso-lts sources compile
 * into the reference binary under oracle/_ref/ (no MPI library exists in this
 * image).  Every collective acts as on a communicator of size 1: reductions
 * and gathers copy, broadcasts and barriers do nothing.  Datatypes are encoded
 * as their byte size so copies know how much to move.
 */
#ifndef MESO_ORACLE_SINGLE_RANK_MPI_H
#define MESO_ORACLE_SINGLE_RANK_MPI_H

#include <cstring>
#include <cstddef>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef std::ptrdiff_t MPI_Aint;
typedef void(MPI_User_function)(void *, void *, int *, MPI_Datatype *);

#define MPI_COMM_WORLD 0
#define MPI_SUM 1
#define MPI_MAX_PROCESSOR_NAME 64
/* datatype handle == element size in bytes */
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_C_BOOL ((MPI_Datatype)sizeof(bool))

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Get_processor_name(char *name, int *len) {
    std::strcpy(name, "single-rank");
    *len = (int)std::strlen(name);
    return 0;
}
inline int MPI_Barrier(MPI_Comm) { return 0; }

/* A struct type is as large as its furthest member end. */
inline int MPI_Type_create_struct(int n, const int *blen, const MPI_Aint *disp,
                                  const MPI_Datatype *types, MPI_Datatype *out) {
    MPI_Aint end = 0;
    for (int i = 0; i < n; ++i) {
        MPI_Aint e = disp[i] + (MPI_Aint)blen[i] * (MPI_Aint)types[i];
        if (e > end) end = e;
    }
    *out = (MPI_Datatype)end;
    return 0;
}
inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
inline int MPI_Type_free(MPI_Datatype *) { return 0; }
inline int MPI_Op_create(MPI_User_function *, int, MPI_Op *op) { *op = MPI_SUM; return 0; }
inline int MPI_Op_free(MPI_Op *) { return 0; }

inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }

inline int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (send != recv && count > 0) std::memmove(recv, send, (size_t)count * (size_t)t);
    return 0;
}

inline int MPI_Gather(const void *send, int scount, MPI_Datatype st, void *recv, int, MPI_Datatype,
                      int, MPI_Comm) {
    if (scount > 0) std::memmove(recv, send, (size_t)scount * (size_t)st);
    return 0;
}

inline int MPI_Gatherv(const void *send, int scount, MPI_Datatype st, void *recv, const int *,
                       const int *displs, MPI_Datatype rt, int, MPI_Comm) {
    if (scount > 0)
        std::memmove((char *)recv + (size_t)displs[0] * (size_t)rt, send, (size_t)scount * (size_t)st);
    return 0;
}

#endif
