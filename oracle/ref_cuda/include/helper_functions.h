/* The CUDA samples' helper_functions.h: nothing of it is used by the compiled
 * reference sources (baseline timing build only). */
#pragma once
