// processorLduInterface.H -- stand-in for OpenFOAM's header of the same name (the class lives
// in lduMatrix.H here).
#include "lduMatrix.H"
