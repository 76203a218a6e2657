// xss_tuning.h -- onesweep pass lines chosen by autotune.py (n = 268435456, _MID classes n = 2097152; uniform keys; median time).
// Each line: BLOCK, ITEMS, MINB, LB, RANK, PERSIST, DPT.
#pragma once
// Every line ranks with RANK 2 (the count atomic's result is the key's rank in
// its warp).  The RANK 0 lines they replace measured, at the same sizes:
// K32 4.18-4.39, K64 12.67, K32V32 7.00, K64V64 17.54, DEFAULT 15.39 ms;
// K32_MID 0.092, K64_MID 0.196, K32V32_MID 0.114, K64V64_MID 0.240,
// DEFAULT_MID 0.228 ms.

// K16 (large 16-bit keys-only arrays sort by counting; this line serves
// chunks of the pipelined host-pointer path): not re-measured with RANK 2
#ifndef XSS_CFG_K16
#define XSS_CFG_K16 320, 20, 3, 16, 2, 1, 0
#endif

// K32 (ranks packed two per register): 320,20,3,8,2,1,0 3.598 ms; 320,24,3,8,2,1,0 3.372 ms; 320,28,2,8,2,1,0 3.738 ms;
// 320,32,2,8,2,1,0 3.513 ms; 320,40,2,8,2,1,0 5.198 ms; 384,32,2,8,2,1,0 3.323 ms; 256,40,2,8,2,1,0 3.788 ms; 256,32,3,8,2,1,0 4.101 ms
// K32 pipelined form (PERSIST 3, resident CTAs holding two tiles), A/B against
// 384,32,2,8,2,1,0 at 2^28: float32 3.586 vs 3.700 ms, uint32 3.293 vs 3.356 ms;
// 384,32,2,8,2,3,0 3.704 / 3.390; 320,20,3,8,2,3,0 3.874 / 3.585; 256,28,3,8,2,3,0 3.671 / 3.372
// One larger CTA per SM (longer tiles, fewer on the look-back chain), float32 / uint32 against
// 3.588 / 3.294: 768,28,1,8,2,3,0 3.807 / 3.520; 768,24,1,8,2,3,0 3.889 / 3.601;
// 640,32,1,8,2,3,0 3.911 / 3.629; 512,40,1,8,2,3,0 4.035 / 3.760; 512,32,1,8,2,3,0 4.222 / 3.946;
// 768,28,1,16,2,3,0 3.883 / 3.606 (two CTAs per SM overlap each other's barrier phases)
#ifndef XSS_CFG_K32
#define XSS_CFG_K32 384, 28, 2, 8, 2, 3, 0
#endif

// K64: 512,16,1,16,2,1,1 10.686 ms; 512,20,1,16,2,1,1 9.931 ms; 512,24,1,16,2,1,1 9.505 ms; 768,16,1,16,2,1,1 10.688 ms
#ifndef XSS_CFG_K64
#define XSS_CFG_K64 512, 24, 1, 16, 2, 1, 1
#endif

// K32V32: 512,14,1,16,2,1,1 5.926 ms; 512,20,1,16,2,1,1 5.173 ms; 768,14,1,16,2,1,1 6.045 ms; 512,24,1,16,2,1,1 4.954 ms
#ifndef XSS_CFG_K32V32
#define XSS_CFG_K32V32 512, 24, 1, 16, 2, 1, 1
#endif

// K64V64: 512,11,1,8,2,1,1 16.375 ms; 512,12,1,8,2,1,1 15.918 ms; 640,10,1,8,2,1,1 15.906 ms; 768,8,1,8,2,1,1 16.529 ms;
// 384,16,1,8,2,1,1 16.101 ms; 512,12,1,16,2,1,1 16.037 ms; 576,11,1,8,2,1,1 15.785 ms
#ifndef XSS_CFG_K64V64
#define XSS_CFG_K64V64 576, 11, 1, 8, 2, 1, 1
#endif

// DEFAULT: 512,14,1,8,2,1,1 13.262 ms; 512,16,1,8,2,1,1 12.557 ms; 640,12,1,8,2,1,1 13.195 ms; 768,10,1,8,2,1,1 13.409 ms;
// 512,17,1,8,2,1,1 12.488 ms
#ifndef XSS_CFG_DEFAULT
#define XSS_CFG_DEFAULT 512, 17, 1, 8, 2, 1, 1
#endif

// K32_MID: 512,16,2,16,2,1,0 0.082 ms; 256,16,3,16,2,1,0 0.093 ms; 256,8,4,16,2,1,0 0.101 ms
#ifndef XSS_CFGM_K32
#define XSS_CFGM_K32 512, 16, 2, 16, 2, 1, 0
#endif

// K64_MID: 512,8,2,16,2,1,1 0.182 ms; 256,16,2,16,2,1,0 0.184 ms
#ifndef XSS_CFGM_K64
#define XSS_CFGM_K64 512, 8, 2, 16, 2, 1, 1
#endif

// K32V32_MID: 512,10,2,16,2,0,0 0.097 ms; 512,10,2,16,2,1,1 0.109 ms
#ifndef XSS_CFGM_K32V32
#define XSS_CFGM_K32V32 512, 10, 2, 16, 2, 0, 0
#endif

// K64V64_MID: 512,6,2,16,2,0,1 0.227 ms; 256,12,2,16,2,0,0 0.238 ms
#ifndef XSS_CFGM_K64V64
#define XSS_CFGM_K64V64 512, 6, 2, 16, 2, 0, 1
#endif

// DEFAULT_MID: 512,6,2,16,2,0,1 0.208 ms; 256,8,3,16,2,0,0 0.212 ms
#ifndef XSS_CFGM_DEFAULT
#define XSS_CFGM_DEFAULT 512, 6, 2, 16, 2, 0, 1
#endif

// K16_MID: 512,16,2,16,2,1,0 0.066 ms; 256,16,3,16,2,1,0 0.066 ms
#ifndef XSS_CFGM_K16
#define XSS_CFGM_K16 256, 16, 3, 16, 2, 1, 0
#endif
