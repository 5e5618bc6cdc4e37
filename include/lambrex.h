// lambrex.h -- drop-in for LAMBReX's lambrex.h (include/lambrex.h:1-9,
// src/lambrex.cpp:4-14): lambrexInit brings up the CUDA device instead of
// amrex::Initialize; lambrexFinalise releases library-wide resources.
#ifndef LAMBREX_H
#define LAMBREX_H

#include "AmrSim.h"

inline void lambrexInit() { lbx::check(lbx_init(), "lambrexInit"); }
inline void lambrexFinalise() { lbx::check(lbx_finalize(), "lambrexFinalise"); }

#endif
