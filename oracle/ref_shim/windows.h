/* Stand-in for <windows.h> so the reference CPU Monte Carlo
 * (monte_cpp/CBCT_real2.cpp:2,87) compiles on Linux: it only uses DWORD. */
#pragma once
typedef unsigned long DWORD;
