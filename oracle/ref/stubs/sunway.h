/* empty stand-in for the Sunway header sunway.h (host-side oracle build) */
