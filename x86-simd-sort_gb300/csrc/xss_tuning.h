// xss_tuning.h -- onesweep pass lines chosen by autotune.py (n = 268435456, uniform keys, median of 5 sorts).
// Each line: BLOCK, ITEMS, MINB, LB, RANK, PERSIST, DPT.
#pragma once

// K16: 512,16,2,16,0,1,0 2.428 ms; 256,24,3,16,0,1,0 2.357 ms; 256,32,2,16,0,1,0 2.516 ms; 256,24,3,16,0,1,1 2.601 ms
#ifndef XSS_CFG_K16
#define XSS_CFG_K16 256, 24, 3, 16, 0, 1, 0
#endif

// K32: 512,16,2,16,0,1,0 4.818 ms; 256,24,3,16,0,1,0 4.730 ms; 256,24,3,16,0,1,1 5.243 ms; 256,32,2,16,0,1,0 4.983 ms; 256,20,3,16,0,1,0 4.973 ms; 512,12,2,16,0,1,1 5.147 ms
#ifndef XSS_CFG_K32
#define XSS_CFG_K32 256, 24, 3, 16, 0, 1, 0
#endif

// K64: 512,8,2,16,0,1,1 13.584 ms; 256,16,2,16,0,1,0 13.526 ms; 512,8,1,16,0,1,1 16.214 ms; 512,10,1,16,0,1,1 14.424 ms
#ifndef XSS_CFG_K64
#define XSS_CFG_K64 256, 16, 2, 16, 0, 1, 0
#endif

// K32V32: 512,10,2,16,0,0,1 7.724 ms; 512,10,2,16,1,0,0 7.973 ms; 512,8,1,16,0,1,1 8.700 ms; 512,10,1,16,1,1,1 8.219 ms
#ifndef XSS_CFG_K32V32
#define XSS_CFG_K32V32 512, 10, 2, 16, 0, 0, 1
#endif

// K64V64: 512,8,1,16,1,1,1 20.098 ms; 512,8,1,16,0,1,1 19.843 ms; 512,6,1,16,1,1,1 23.240 ms; 512,10,1,16,1,1,1 18.495 ms; 256,12,2,16,1,0,0 21.481 ms
#ifndef XSS_CFG_K64V64
#define XSS_CFG_K64V64 512, 10, 1, 16, 1, 1, 1
#endif

// DEFAULT: 512,6,2,16,0,0,1 20.209 ms; 512,8,1,16,0,1,1 18.748 ms; 512,8,1,16,1,1,1 19.397 ms; 256,12,2,16,1,0,0 20.582 ms
#ifndef XSS_CFG_DEFAULT
#define XSS_CFG_DEFAULT 512, 8, 1, 16, 0, 1, 1
#endif
