// xss_tuning.h -- onesweep pass lines chosen by autotune.py (n = 268435456, _MID classes n = 2097152; uniform keys; median time).
// Each line: BLOCK, ITEMS, MINB, LB, RANK, PERSIST, DPT.
#pragma once
// Look-back width re-measured afterwards (autotune.py --candidates): LB 8 beat LB 16 for
// K32 (4.255 vs 4.331 ms), K64V64 (17.33 vs 17.49 ms) and DEFAULT (15.23 vs 15.35 ms);
// those three lines use it.  K32 with the keys-only first pass ranking tie-free, uint32
// keys at 2^28: LB 8 4.183 ms, LB 4 4.208, LB 32 4.758; look-back started early on 128
// threads x 2 digits (DPT 2) 4.821, on 64 threads x 4 digits (DPT 4) 5.626 ms.

// K16: 320,20,3,16,0,1,0 2.153 ms; 256,24,3,16,0,1,0 2.273 ms; 512,16,2,16,0,1,0 2.252 ms
#ifndef XSS_CFG_K16
#define XSS_CFG_K16 320, 20, 3, 16, 0, 1, 0
#endif

// K32: 320,20,3,16,0,1,0 4.389 ms; 256,24,3,16,0,1,0 4.605 ms; 512,16,2,16,0,1,0 4.532 ms; 320,24,2,16,0,1,0 4.816 ms
#ifndef XSS_CFG_K32
#define XSS_CFG_K32 320, 20, 3, 8, 0, 1, 0
#endif

// K64: 512,16,1,16,0,1,1 12.669 ms; 512,12,1,16,0,1,1 13.474 ms; 256,16,2,16,0,1,0 13.229 ms
#ifndef XSS_CFG_K64
#define XSS_CFG_K64 512, 16, 1, 16, 0, 1, 1
#endif

// K32V32: 512,12,1,16,0,1,1 7.319 ms; 512,10,2,16,0,0,1 7.644 ms; 512,14,1,16,0,1,1 6.999 ms
#ifndef XSS_CFG_K32V32
#define XSS_CFG_K32V32 512, 14, 1, 16, 0, 1, 1
#endif

// K64V64: 512,11,1,16,1,1,1 17.939 ms; 512,11,1,16,0,1,1 17.538 ms; 512,10,1,16,0,1,1 18.100 ms; 512,12,1,16,0,1,1 inf ms
#ifndef XSS_CFG_K64V64
#define XSS_CFG_K64V64 512, 11, 1, 8, 0, 1, 1
#endif

// DEFAULT: 512,14,1,16,0,1,1 15.387 ms; 512,12,1,16,0,1,1 15.975 ms; 512,14,1,16,1,1,1 17.137 ms
#ifndef XSS_CFG_DEFAULT
#define XSS_CFG_DEFAULT 512, 14, 1, 8, 0, 1, 1
#endif

// K16_MID: 512,16,2,16,0,1,0 0.057 ms; 256,16,3,16,0,1,0 0.060 ms
#ifndef XSS_CFGM_K16
#define XSS_CFGM_K16 512, 16, 2, 16, 0, 1, 0
#endif

// K32_MID: 512,16,2,16,0,1,0 0.092 ms; 256,16,3,16,0,1,0 0.100 ms; 512,8,2,16,0,0,1 0.100 ms
#ifndef XSS_CFGM_K32
#define XSS_CFGM_K32 512, 16, 2, 16, 0, 1, 0
#endif

// K64_MID: 512,8,2,16,0,1,1 0.196 ms; 256,16,2,16,1,1,0 0.198 ms; 256,16,2,16,0,1,0 0.199 ms
#ifndef XSS_CFGM_K64
#define XSS_CFGM_K64 512, 8, 2, 16, 0, 1, 1
#endif

// K32V32_MID: 512,10,2,16,1,0,0 0.115 ms; 512,10,2,16,0,0,0 0.114 ms; 512,6,2,16,1,0,1 0.119 ms
#ifndef XSS_CFGM_K32V32
#define XSS_CFGM_K32V32 512, 10, 2, 16, 0, 0, 0
#endif

// K64V64_MID: 512,6,2,16,1,0,1 0.242 ms; 512,6,2,16,0,0,1 0.240 ms; 256,12,2,16,1,0,0 0.246 ms
#ifndef XSS_CFGM_K64V64
#define XSS_CFGM_K64V64 512, 6, 2, 16, 0, 0, 1
#endif

// DEFAULT_MID: 512,6,2,16,0,0,1 0.228 ms; 256,12,2,16,1,0,0 0.235 ms; 256,8,3,16,1,0,0 0.228 ms
#ifndef XSS_CFGM_DEFAULT
#define XSS_CFGM_DEFAULT 512, 6, 2, 16, 0, 0, 1
#endif
