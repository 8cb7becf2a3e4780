// batched.cuh -- ragged batches of small LU solves (C entry points in tmvg.h).
#pragma once

#include "common.cuh"
