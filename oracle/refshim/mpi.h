/* Single-rank stand-in for the MPI calls cajitafluids' headers make
 * (oracle reference pin): one rank, rank 0. */
#ifndef CFREF_MPI_H
#define CFREF_MPI_H
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
static inline int MPI_Comm_rank(MPI_Comm, int* rank) {
    *rank = 0;
    return 0;
}
static inline int MPI_Comm_size(MPI_Comm, int* size) {
    *size = 1;
    return 0;
}
#endif
