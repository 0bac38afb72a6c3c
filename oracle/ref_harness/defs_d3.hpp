// TEST INFRASTRUCTURE ONLY: problem definitions of the 3-D reference build
// (as test/MHD/OrszagTang3D/definitions.hpp)
#define COMPONENTS 3
#define DIMENSIONS 3
#define GEOMETRY CARTESIAN
