// Test infrastructure only: every vector stand-in at once, as SEP's own
// headers make them visible to one another.
#pragma once
#include "float1DReg.h"
#include "float2DReg.h"
#include "float3DReg.h"
#include "float4DReg.h"
#include "complex1DReg.h"
#include "complex2DReg.h"
#include "complex3DReg.h"
#include "complex4DReg.h"
