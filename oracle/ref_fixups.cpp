// ref_fixups.cpp -- link-time stand-ins for two reference functions whose bodies have
// undefined behaviour under a current compiler.  TEST INFRASTRUCTURE ONLY (part of
// oracle/_ref/cgppd_ref_mc).
//
// src/vector3f.cpp:105-117 declares Vector3f::operator+= and operator-= to return a
// Vector3f but has no return statement.  Every caller discards the value (e.g.
// src/Molecule.cpp:280-299); the compilers the reference was built with let control
// fall off the end, but g++ 13 treats that path as unreachable (at -O2 the function runs
// into the next one; at -O0 it traps).  The MC harness is linked with
// -Wl,--wrap for both symbols, so every call from another file reaches these
// definitions: the same float component updates, then the updated vector is returned.
#include "vector3f.h"

extern "C" Vector3f __wrap__ZN8Vector3fpLES_(Vector3f *self, Vector3f v)
{
    self->x = self->x + v.x;
    self->y = self->y + v.y;
    self->z = self->z + v.z;
    return *self;
}

extern "C" Vector3f __wrap__ZN8Vector3fmIES_(Vector3f *self, Vector3f v)
{
    self->x = self->x - v.x;
    self->y = self->y - v.y;
    self->z = self->z - v.z;
    return *self;
}
