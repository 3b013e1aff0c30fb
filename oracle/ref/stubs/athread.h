/* empty stand-in for the Sunway header athread.h (host-side oracle build) */
#define SLAVE_FUN(f) slave_##f
static inline int athread_idle(void) { return 1; }
static inline int athread_init(void) { return 0; }
#define athread_spawn(f, a) ((void)(a), 0)
#define athread_join() 0
