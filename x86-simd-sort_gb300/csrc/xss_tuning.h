// xss_tuning.h -- onesweep pass lines chosen by autotune.py (n = 268435456, uniform keys, median of 5 sorts).
// Each line: BLOCK, ITEMS, MINB, LB, RANK, PERSIST, DPT.
#pragma once

// K16: 256,24,3,16,0,1,0 2.360 ms; 512,16,2,16,0,1,0 2.427 ms; 320,20,3,16,0,1,0 2.309 ms
#ifndef XSS_CFG_K16
#define XSS_CFG_K16 320, 20, 3, 16, 0, 1, 0
#endif

// K32: 320,20,3,16,0,1,0 4.648 ms; 256,24,3,16,0,1,0 4.732 ms; 512,16,2,16,0,1,0 4.819 ms; 384,16,3,16,0,1,0 5.252 ms
#ifndef XSS_CFG_K32
#define XSS_CFG_K32 320, 20, 3, 16, 0, 1, 0
#endif

// K64: 256,16,2,16,0,1,0 13.416 ms; 512,12,1,16,0,1,1 13.400 ms; 512,16,1,16,0,1,1 12.773 ms; 512,8,2,16,0,1,1 13.602 ms
#ifndef XSS_CFG_K64
#define XSS_CFG_K64 512, 16, 1, 16, 0, 1, 1
#endif

// K32V32: 512,10,2,16,0,0,1 7.852 ms; 512,12,1,16,0,1,1 7.349 ms; 512,14,1,16,1,1,1 7.499 ms
#ifndef XSS_CFG_K32V32
#define XSS_CFG_K32V32 512, 12, 1, 16, 0, 1, 1
#endif

// K64V64: 512,11,1,16,1,1,1 18.000 ms; 512,12,1,16,1,1,1 19.056 ms; 512,10,1,16,0,1,1 18.231 ms; 512,6,2,16,1,0,1 21.274 ms
#ifndef XSS_CFG_K64V64
#define XSS_CFG_K64V64 512, 11, 1, 16, 1, 1, 1
#endif

// DEFAULT: 512,12,1,16,0,1,1 16.129 ms; 512,14,1,16,0,1,1 15.672 ms; 512,12,1,16,1,1,1 16.723 ms; 512,6,2,16,0,0,1 20.688 ms
#ifndef XSS_CFG_DEFAULT
#define XSS_CFG_DEFAULT 512, 14, 1, 16, 0, 1, 1
#endif

// mid-size classes
// K16_MID: 512,16,2,16,0,1,0 0.056 ms; 256,16,3,16,0,1,0 0.060 ms; 256,8,4,16,0,0,0 0.066 ms
#ifndef XSS_CFGM_K16
#define XSS_CFGM_K16 512, 16, 2, 16, 0, 1, 0
#endif

// K32_MID: 512,16,2,16,0,1,0 0.093 ms; 256,16,3,16,0,1,0 0.101 ms; 256,8,4,16,0,0,0 0.109 ms; 512,8,2,16,0,0,1 0.100 ms; 320,20,3,16,0,1,0 0.107 ms
#ifndef XSS_CFGM_K32
#define XSS_CFGM_K32 512, 16, 2, 16, 0, 1, 0
#endif

// K64_MID: 256,16,2,16,1,1,0 0.198 ms; 256,8,3,16,1,0,0 0.204 ms; 512,8,2,16,0,1,1 0.197 ms
#ifndef XSS_CFGM_K64
#define XSS_CFGM_K64 512, 8, 2, 16, 0, 1, 1
#endif

// K32V32_MID: 512,10,2,16,1,0,0 0.114 ms; 256,8,3,16,1,0,0 0.119 ms; 512,6,2,16,1,0,1 0.117 ms
#ifndef XSS_CFGM_K32V32
#define XSS_CFGM_K32V32 512, 10, 2, 16, 1, 0, 0
#endif

// K64V64_MID: 256,12,2,16,1,0,0 0.250 ms; 256,6,3,16,1,0,0 0.261 ms; 512,6,2,16,1,0,1 0.246 ms
#ifndef XSS_CFGM_K64V64
#define XSS_CFGM_K64V64 512, 6, 2, 16, 1, 0, 1
#endif

// DEFAULT_MID: 256,12,2,16,1,0,0 0.238 ms; 512,6,2,16,0,0,1 0.227 ms; 256,8,3,16,1,0,0 0.231 ms
#ifndef XSS_CFGM_DEFAULT
#define XSS_CFGM_DEFAULT 512, 6, 2, 16, 0, 0, 1
#endif
