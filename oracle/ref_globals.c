/*
 * Defines the reference's global state the way its evp.c does (evp.c:1-4):
 * by including the reference's evp.h with EVP_GLOBALS_ONCE set.
 * TEST INFRASTRUCTURE ONLY (part of the oracle/_ref build).
 */
#define EVP_GLOBALS_ONCE
#include "evp.h"
#undef EVP_GLOBALS_ONCE
