/* Tree depth of the reference's CPU FMM, set by oracle/rtfmm_driver.cpp (the
 * reference fixes it to 3 at fmm.cpp:21).  TEST INFRASTRUCTURE ONLY. */
#pragma once
extern "C" int rtfmm_depth();
