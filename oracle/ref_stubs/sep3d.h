/* Stand-in for SEPlib's sep3d.h (see seplib.h in this folder). */
#ifndef SEPX_REF_SEP3D_STUB_H
#define SEPX_REF_SEP3D_STUB_H
#include "seplib.h"
#endif
