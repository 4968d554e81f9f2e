/* Test infrastructure for the oracle: the reference's kernels are compiled as plain
 * host functions; the launch coordinates they read are the thread-local globals
 * declared in cpt_ref_prelude.h. */
#pragma once
