/* same single-process MPI stand-ins as ../mpi.h */
#include "../mpi.h"
