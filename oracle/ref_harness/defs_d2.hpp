// TEST INFRASTRUCTURE ONLY: problem definitions of the 2-D reference build
// (as test/MHD/OrszagTang/definitions.hpp)
#define COMPONENTS 2
#define DIMENSIONS 2
#define GEOMETRY CARTESIAN
