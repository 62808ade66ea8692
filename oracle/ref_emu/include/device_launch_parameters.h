#pragma once
/* threadIdx/blockIdx/blockDim/gridDim are declared in emu_prelude.h */
