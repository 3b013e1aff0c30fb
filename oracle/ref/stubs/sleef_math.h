/* empty stand-in for the Sunway header sleef_math.h (host-side oracle build) */
