// Stand-in for SEP genericIO's ioModes.h (test infrastructure only): no I/O
// modes; it brings in the vector and parameter stand-ins the reference's
// headers expect to arrive through it.
#pragma once
#include "complex4DReg.h"
#include "floatHyper.h"
#include "json/json.h"
#include "paramObj.h"
