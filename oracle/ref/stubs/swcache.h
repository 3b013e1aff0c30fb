/* empty stand-in for the Sunway header swcache.h (host-side oracle build) */
