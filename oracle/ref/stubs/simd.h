/* empty stand-in for the Sunway header simd.h (host-side oracle build) */
typedef double doublev4 __attribute__((vector_size(32)));
typedef int intv8 __attribute__((vector_size(32)));
