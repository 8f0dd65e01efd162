/*
 * Single-process stand-in for the MPI names that the reference's init.c,
 * allvars.c and gridding.c use (test infrastructure: used only to compile the
 * reference's own reader, sectoring, gridding loop and grid dump writer into
 * oracle/_ref/refio).  With one process:
 *   - broadcasts, barriers, fences and window locks do nothing;
 *   - MPI_Reduce of one contribution copies the send buffer to the receive
 *     buffer (the reference reduces doubles only);
 *   - MPI_Get reads from the base of the window that MPI_Win_create
 *     registered (the reference gets doubles only, from rank 0 here).
 * No MPI library is involved.
 */
#ifndef WSTACK_ORACLE_REFSHIM_MPI_H_
#define WSTACK_ORACLE_REFSHIM_MPI_H_
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Win;
typedef long MPI_Aint;
typedef int MPI_Request;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_BYTE 0
#define MPI_DOUBLE 1
#define MPI_SUM 0
#define MPI_INFO_NULL 0
#define MPI_LOCK_SHARED 0
#define MPI_Bcast(...) 0
#define MPI_Barrier(...) 0
#define MPI_Wtime() 0.0
#define MPI_Win_fence(...) 0
#define MPI_Win_lock(...) 0
#define MPI_Win_unlock(...) 0
#define MPI_Win_free(...) 0

static void *refshim_win_base[16];
static int refshim_nwin;
static inline int refshim_win_create(void *base, MPI_Win *win)
{
    refshim_win_base[refshim_nwin & 15] = base;
    *win = refshim_nwin++ & 15;
    return 0;
}
#define MPI_Win_create(base, size, disp, info, comm, win) refshim_win_create((base), (win))
#define MPI_Get(origin, ocount, otype, target, disp, tcount, ttype, win)                    \
    (memcpy((origin), (const double *)refshim_win_base[(win)] + (disp),                      \
            (size_t)(ocount) * sizeof(double)), 0)
#define MPI_Reduce(sbuf, rbuf, count, type, op, root, comm)                                 \
    ((const void *)(sbuf) != (const void *)(rbuf)                                          \
         ? (memcpy((rbuf), (sbuf), (size_t)(count) * sizeof(double)), 0) : 0)
#endif
