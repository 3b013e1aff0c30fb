/* empty stand-in for the Sunway header gptl.h (host-side oracle build) */
#define GPTLstart(x) 0
#define GPTLstop(x) 0
