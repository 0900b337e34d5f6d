// Generated by gen_mt_tables.py from the Dax marching-tetrahedra case table
// (dax/worklet/internal/MarchingTetrahedraTable.h:28-53). Do not edit.
// Word layout: bits 4n..4n+3 = edge of output vertex n (0xF unused),
// bits 28..31 = triangle count of the case.
#pragma once
#include <stdint.h>
#define DAX_GB300_MT_CASE_WORDS { \
  0x00ffffffu, 0x10fff230u, 0x10fff410u, 0x20231341u, \
  0x10fff521u, 0x20531130u, 0x20420452u, 0x10fff453u, \
  0x10fff543u, 0x20542402u, 0x20350510u, 0x10fff251u, \
  0x20213143u, 0x10fff140u, 0x10fff320u, 0x00ffffffu \
}
