// Stand-in for the psi4 header of the same path: everything the ugacc hot-path
// sources need from psi4 is declared once in psi4_shim.h.
#pragma once
#include "../../psi4_shim.h"
