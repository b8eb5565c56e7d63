// Pstream.H -- stand-in for OpenFOAM's header of the same name (the parallel-run classes
// live in lduMatrix.H here).
#include "lduMatrix.H"
