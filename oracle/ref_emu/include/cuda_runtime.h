#pragma once
#include "cuda_runtime_api.h"
#include "vector_types.h"
#include "vector_functions.h"
