/*
 * Single-process stand-in for the MPI names that the reference's init.c and
 * allvars.c mention (test infrastructure: used only to compile the
 * reference's own reader into oracle/_ref/refio).  With one rank every
 * broadcast and barrier in those files is a no-op, which is what these macros
 * make them.  No MPI library is involved.
 */
#ifndef WSTACK_ORACLE_REFSHIM_MPI_H_
#define WSTACK_ORACLE_REFSHIM_MPI_H_
typedef int MPI_Comm;
typedef int MPI_Win;
typedef long MPI_Aint;
typedef int MPI_Request;
typedef int MPI_Datatype;
#define MPI_COMM_WORLD 0
#define MPI_BYTE 0
#define MPI_Bcast(...) 0
#define MPI_Barrier(...) 0
#define MPI_Wtime() 0.0
#endif
