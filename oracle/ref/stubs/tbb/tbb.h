// Stand-in for TBB (test infrastructure only).
#pragma once
#include "blocked_range.h"
#include "blocked_range2d.h"
#include "cache_aligned_allocator.h"
#include "global_control.h"
#include "mutex.h"
#include "parallel_for.h"
#include "parallel_reduce.h"
