#pragma once
// Intentionally empty: replaced by curand_kernel.h in this directory.
