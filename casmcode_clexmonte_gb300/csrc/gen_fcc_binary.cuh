// GENERATED by casmcode_clexmonte_gb300/codegen.py -- do not edit.
// Site evaluator of the binary FCC cluster expansion: point, pairs to the
// third neighbour shell, triplets with all edges up to the second shell.
#pragma once
#include <cstdint>
namespace cem {
namespace gen_fcc {
constexpr int N_NB = 42;
constexpr int N_ORBITS = 6;
constexpr int ORBIT_SIZE[N_ORBITS] = {1, 2, 2, 2, 3, 3};
constexpr int ORBIT_CLUSTERS[N_ORBITS] = {1, 12, 6, 24, 24, 36};
// neighbour cell offsets (dx, dy, dz)
constexpr int NB[N_NB][3] = {
    {-1, 0, 0}, {-1, 0, 1}, {-1, 1, 0}, {0, -1, 0}, {0, -1, 1}, {0, 0, -1}, {0, 0, 1}, {0, 1, -1}, {0, 1, 0}, {1, -1, 0}, {1, 0, -1}, {1, 0, 0}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, -1, -1}, {1, -1, 1}, {1, 1, -1}, {-2, 0, 1}, {-2, 1, 0}, {-2, 1, 1}, {-1, -1, 0}, {-1, -1, 2}, {-1, 0, -1}, {-1, 0, 2}, {-1, 2, -1}, {-1, 2, 0}, {0, -2, 1}, {0, -1, -1}, {0, -1, 2}, {0, 1, -2}, {0, 1, 1}, {0, 2, -1}, {1, -2, 0}, {1, -2, 1}, {1, 0, -2}, {1, 0, 1}, {1, 1, -2}, {1, 1, 0}, {2, -1, -1}, {2, -1, 0}, {2, 0, -1}};
// per orbit: partner neighbour indices of every flower cluster
constexpr int N_CL = 103;
constexpr int CL_ORBIT[N_CL] = {0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5};
constexpr int CL_P[N_CL][3] = {{-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {2, -1, -1}, {3, -1, -1}, {4, -1, -1}, {5, -1, -1}, {6, -1, -1}, {7, -1, -1}, {8, -1, -1}, {9, -1, -1}, {10, -1, -1}, {11, -1, -1}, {12, -1, -1}, {13, -1, -1}, {14, -1, -1}, {15, -1, -1}, {16, -1, -1}, {17, -1, -1}, {18, -1, -1}, {19, -1, -1}, {20, -1, -1}, {21, -1, -1}, {22, -1, -1}, {23, -1, -1}, {24, -1, -1}, {25, -1, -1}, {26, -1, -1}, {27, -1, -1}, {28, -1, -1}, {29, -1, -1}, {30, -1, -1}, {31, -1, -1}, {32, -1, -1}, {33, -1, -1}, {34, -1, -1}, {35, -1, -1}, {36, -1, -1}, {37, -1, -1}, {38, -1, -1}, {39, -1, -1}, {40, -1, -1}, {41, -1, -1}, {0, 1, -1}, {0, 2, -1}, {0, 3, -1}, {0, 5, -1}, {1, 2, -1}, {1, 4, -1}, {1, 6, -1}, {2, 7, -1}, {2, 8, -1}, {3, 4, -1}, {3, 5, -1}, {3, 9, -1}, {4, 6, -1}, {4, 9, -1}, {5, 7, -1}, {5, 10, -1}, {6, 8, -1}, {6, 11, -1}, {7, 8, -1}, {7, 10, -1}, {8, 11, -1}, {9, 10, -1}, {9, 11, -1}, {10, 11, -1}, {12, 0, -1}, {12, 1, -1}, {12, 3, -1}, {12, 4, -1}, {0, 13, -1}, {0, 4, -1}, {0, 7, -1}, {1, 14, -1}, {1, 3, -1}, {1, 8, -1}, {13, 2, -1}, {13, 5, -1}, {13, 7, -1}, {2, 14, -1}, {2, 5, -1}, {2, 6, -1}, {14, 6, -1}, {14, 8, -1}, {3, 15, -1}, {3, 10, -1}, {4, 16, -1}, {4, 11, -1}, {5, 15, -1}, {5, 9, -1}, {6, 9, -1}, {6, 16, -1}, {7, 11, -1}, {7, 17, -1}, {8, 10, -1}, {8, 17, -1}, {15, 9, -1}, {15, 10, -1}, {9, 16, -1}, {16, 11, -1}, {10, 17, -1}, {11, 17, -1}};
// copies in constant memory for run-time indexing on the device
static __constant__ int NB_D[N_NB][3] = {
    {-1, 0, 0}, {-1, 0, 1}, {-1, 1, 0}, {0, -1, 0}, {0, -1, 1}, {0, 0, -1}, {0, 0, 1}, {0, 1, -1}, {0, 1, 0}, {1, -1, 0}, {1, 0, -1}, {1, 0, 0}, {-1, -1, 1}, {-1, 1, -1}, {-1, 1, 1}, {1, -1, -1}, {1, -1, 1}, {1, 1, -1}, {-2, 0, 1}, {-2, 1, 0}, {-2, 1, 1}, {-1, -1, 0}, {-1, -1, 2}, {-1, 0, -1}, {-1, 0, 2}, {-1, 2, -1}, {-1, 2, 0}, {0, -2, 1}, {0, -1, -1}, {0, -1, 2}, {0, 1, -2}, {0, 1, 1}, {0, 2, -1}, {1, -2, 0}, {1, -2, 1}, {1, 0, -2}, {1, 0, 1}, {1, 1, -2}, {1, 1, 0}, {2, -1, -1}, {2, -1, 0}, {2, 0, -1}};
static __constant__ int CL_ORBIT_D[N_CL] = {0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5};
static __constant__ int CL_P_D[N_CL][3] = {{-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {2, -1, -1}, {3, -1, -1}, {4, -1, -1}, {5, -1, -1}, {6, -1, -1}, {7, -1, -1}, {8, -1, -1}, {9, -1, -1}, {10, -1, -1}, {11, -1, -1}, {12, -1, -1}, {13, -1, -1}, {14, -1, -1}, {15, -1, -1}, {16, -1, -1}, {17, -1, -1}, {18, -1, -1}, {19, -1, -1}, {20, -1, -1}, {21, -1, -1}, {22, -1, -1}, {23, -1, -1}, {24, -1, -1}, {25, -1, -1}, {26, -1, -1}, {27, -1, -1}, {28, -1, -1}, {29, -1, -1}, {30, -1, -1}, {31, -1, -1}, {32, -1, -1}, {33, -1, -1}, {34, -1, -1}, {35, -1, -1}, {36, -1, -1}, {37, -1, -1}, {38, -1, -1}, {39, -1, -1}, {40, -1, -1}, {41, -1, -1}, {0, 1, -1}, {0, 2, -1}, {0, 3, -1}, {0, 5, -1}, {1, 2, -1}, {1, 4, -1}, {1, 6, -1}, {2, 7, -1}, {2, 8, -1}, {3, 4, -1}, {3, 5, -1}, {3, 9, -1}, {4, 6, -1}, {4, 9, -1}, {5, 7, -1}, {5, 10, -1}, {6, 8, -1}, {6, 11, -1}, {7, 8, -1}, {7, 10, -1}, {8, 11, -1}, {9, 10, -1}, {9, 11, -1}, {10, 11, -1}, {12, 0, -1}, {12, 1, -1}, {12, 3, -1}, {12, 4, -1}, {0, 13, -1}, {0, 4, -1}, {0, 7, -1}, {1, 14, -1}, {1, 3, -1}, {1, 8, -1}, {13, 2, -1}, {13, 5, -1}, {13, 7, -1}, {2, 14, -1}, {2, 5, -1}, {2, 6, -1}, {14, 6, -1}, {14, 8, -1}, {3, 15, -1}, {3, 10, -1}, {4, 16, -1}, {4, 11, -1}, {5, 15, -1}, {5, 9, -1}, {6, 9, -1}, {6, 16, -1}, {7, 11, -1}, {7, 17, -1}, {8, 10, -1}, {8, 17, -1}, {15, 9, -1}, {15, 10, -1}, {9, 16, -1}, {16, 11, -1}, {10, 17, -1}, {11, 17, -1}};

// counts[g] = number of clusters of orbit g whose partners are all 1
template <int P>
__device__ __forceinline__ void counts(const int8_t *__restrict__ c, int (&n)[N_ORBITS]) {
  const int v0 = c[(-1) + P * (0) + P * P * (0)];
  const int v1 = c[(-1) + P * (0) + P * P * (1)];
  const int v2 = c[(-1) + P * (1) + P * P * (0)];
  const int v3 = c[(0) + P * (-1) + P * P * (0)];
  const int v4 = c[(0) + P * (-1) + P * P * (1)];
  const int v5 = c[(0) + P * (0) + P * P * (-1)];
  const int v6 = c[(0) + P * (0) + P * P * (1)];
  const int v7 = c[(0) + P * (1) + P * P * (-1)];
  const int v8 = c[(0) + P * (1) + P * P * (0)];
  const int v9 = c[(1) + P * (-1) + P * P * (0)];
  const int v10 = c[(1) + P * (0) + P * P * (-1)];
  const int v11 = c[(1) + P * (0) + P * P * (0)];
  const int v12 = c[(-1) + P * (-1) + P * P * (1)];
  const int v13 = c[(-1) + P * (1) + P * P * (-1)];
  const int v14 = c[(-1) + P * (1) + P * P * (1)];
  const int v15 = c[(1) + P * (-1) + P * P * (-1)];
  const int v16 = c[(1) + P * (-1) + P * P * (1)];
  const int v17 = c[(1) + P * (1) + P * P * (-1)];
  const int v18 = c[(-2) + P * (0) + P * P * (1)];
  const int v19 = c[(-2) + P * (1) + P * P * (0)];
  const int v20 = c[(-2) + P * (1) + P * P * (1)];
  const int v21 = c[(-1) + P * (-1) + P * P * (0)];
  const int v22 = c[(-1) + P * (-1) + P * P * (2)];
  const int v23 = c[(-1) + P * (0) + P * P * (-1)];
  const int v24 = c[(-1) + P * (0) + P * P * (2)];
  const int v25 = c[(-1) + P * (2) + P * P * (-1)];
  const int v26 = c[(-1) + P * (2) + P * P * (0)];
  const int v27 = c[(0) + P * (-2) + P * P * (1)];
  const int v28 = c[(0) + P * (-1) + P * P * (-1)];
  const int v29 = c[(0) + P * (-1) + P * P * (2)];
  const int v30 = c[(0) + P * (1) + P * P * (-2)];
  const int v31 = c[(0) + P * (1) + P * P * (1)];
  const int v32 = c[(0) + P * (2) + P * P * (-1)];
  const int v33 = c[(1) + P * (-2) + P * P * (0)];
  const int v34 = c[(1) + P * (-2) + P * P * (1)];
  const int v35 = c[(1) + P * (0) + P * P * (-2)];
  const int v36 = c[(1) + P * (0) + P * P * (1)];
  const int v37 = c[(1) + P * (1) + P * P * (-2)];
  const int v38 = c[(1) + P * (1) + P * P * (0)];
  const int v39 = c[(2) + P * (-1) + P * P * (-1)];
  const int v40 = c[(2) + P * (-1) + P * P * (0)];
  const int v41 = c[(2) + P * (0) + P * P * (-1)];
  n[0] = 1;
  n[1] = v0 + v1 + v2 + v3 + v4 + v5 + v6 + v7 + v8 + v9 + v10 + v11;
  n[2] = v12 + v13 + v14 + v15 + v16 + v17;
  n[3] = v18 + v19 + v20 + v21 + v22 + v23 + v24 + v25 + v26 + v27 + v28 + v29 + v30 + v31 + v32 + v33 + v34 + v35 + v36 + v37 + v38 + v39 + v40 + v41;
  n[4] = (v0 & v1) + (v0 & v2) + (v0 & v3) + (v0 & v5) + (v1 & v2) + (v1 & v4) + (v1 & v6) + (v2 & v7) + (v2 & v8) + (v3 & v4) + (v3 & v5) + (v3 & v9) + (v4 & v6) + (v4 & v9) + (v5 & v7) + (v5 & v10) + (v6 & v8) + (v6 & v11) + (v7 & v8) + (v7 & v10) + (v8 & v11) + (v9 & v10) + (v9 & v11) + (v10 & v11);
  n[5] = (v12 & v0) + (v12 & v1) + (v12 & v3) + (v12 & v4) + (v0 & v13) + (v0 & v4) + (v0 & v7) + (v1 & v14) + (v1 & v3) + (v1 & v8) + (v13 & v2) + (v13 & v5) + (v13 & v7) + (v2 & v14) + (v2 & v5) + (v2 & v6) + (v14 & v6) + (v14 & v8) + (v3 & v15) + (v3 & v10) + (v4 & v16) + (v4 & v11) + (v5 & v15) + (v5 & v9) + (v6 & v9) + (v6 & v16) + (v7 & v11) + (v7 & v17) + (v8 & v10) + (v8 & v17) + (v15 & v9) + (v15 & v10) + (v9 & v16) + (v16 & v11) + (v10 & v17) + (v11 & v17);
}

// the same counts, and the neighbour occupants packed into env (bit k =
// neighbour k), the input of the proposal network
template <int P>
__device__ __forceinline__ void counts_env(const int8_t *__restrict__ c, int (&n)[N_ORBITS],
                                           unsigned long long &env) {
  const int v0 = c[(-1) + P * (0) + P * P * (0)];
  const int v1 = c[(-1) + P * (0) + P * P * (1)];
  const int v2 = c[(-1) + P * (1) + P * P * (0)];
  const int v3 = c[(0) + P * (-1) + P * P * (0)];
  const int v4 = c[(0) + P * (-1) + P * P * (1)];
  const int v5 = c[(0) + P * (0) + P * P * (-1)];
  const int v6 = c[(0) + P * (0) + P * P * (1)];
  const int v7 = c[(0) + P * (1) + P * P * (-1)];
  const int v8 = c[(0) + P * (1) + P * P * (0)];
  const int v9 = c[(1) + P * (-1) + P * P * (0)];
  const int v10 = c[(1) + P * (0) + P * P * (-1)];
  const int v11 = c[(1) + P * (0) + P * P * (0)];
  const int v12 = c[(-1) + P * (-1) + P * P * (1)];
  const int v13 = c[(-1) + P * (1) + P * P * (-1)];
  const int v14 = c[(-1) + P * (1) + P * P * (1)];
  const int v15 = c[(1) + P * (-1) + P * P * (-1)];
  const int v16 = c[(1) + P * (-1) + P * P * (1)];
  const int v17 = c[(1) + P * (1) + P * P * (-1)];
  const int v18 = c[(-2) + P * (0) + P * P * (1)];
  const int v19 = c[(-2) + P * (1) + P * P * (0)];
  const int v20 = c[(-2) + P * (1) + P * P * (1)];
  const int v21 = c[(-1) + P * (-1) + P * P * (0)];
  const int v22 = c[(-1) + P * (-1) + P * P * (2)];
  const int v23 = c[(-1) + P * (0) + P * P * (-1)];
  const int v24 = c[(-1) + P * (0) + P * P * (2)];
  const int v25 = c[(-1) + P * (2) + P * P * (-1)];
  const int v26 = c[(-1) + P * (2) + P * P * (0)];
  const int v27 = c[(0) + P * (-2) + P * P * (1)];
  const int v28 = c[(0) + P * (-1) + P * P * (-1)];
  const int v29 = c[(0) + P * (-1) + P * P * (2)];
  const int v30 = c[(0) + P * (1) + P * P * (-2)];
  const int v31 = c[(0) + P * (1) + P * P * (1)];
  const int v32 = c[(0) + P * (2) + P * P * (-1)];
  const int v33 = c[(1) + P * (-2) + P * P * (0)];
  const int v34 = c[(1) + P * (-2) + P * P * (1)];
  const int v35 = c[(1) + P * (0) + P * P * (-2)];
  const int v36 = c[(1) + P * (0) + P * P * (1)];
  const int v37 = c[(1) + P * (1) + P * P * (-2)];
  const int v38 = c[(1) + P * (1) + P * P * (0)];
  const int v39 = c[(2) + P * (-1) + P * P * (-1)];
  const int v40 = c[(2) + P * (-1) + P * P * (0)];
  const int v41 = c[(2) + P * (0) + P * P * (-1)];
  n[0] = 1;
  n[1] = v0 + v1 + v2 + v3 + v4 + v5 + v6 + v7 + v8 + v9 + v10 + v11;
  n[2] = v12 + v13 + v14 + v15 + v16 + v17;
  n[3] = v18 + v19 + v20 + v21 + v22 + v23 + v24 + v25 + v26 + v27 + v28 + v29 + v30 + v31 + v32 + v33 + v34 + v35 + v36 + v37 + v38 + v39 + v40 + v41;
  n[4] = (v0 & v1) + (v0 & v2) + (v0 & v3) + (v0 & v5) + (v1 & v2) + (v1 & v4) + (v1 & v6) + (v2 & v7) + (v2 & v8) + (v3 & v4) + (v3 & v5) + (v3 & v9) + (v4 & v6) + (v4 & v9) + (v5 & v7) + (v5 & v10) + (v6 & v8) + (v6 & v11) + (v7 & v8) + (v7 & v10) + (v8 & v11) + (v9 & v10) + (v9 & v11) + (v10 & v11);
  n[5] = (v12 & v0) + (v12 & v1) + (v12 & v3) + (v12 & v4) + (v0 & v13) + (v0 & v4) + (v0 & v7) + (v1 & v14) + (v1 & v3) + (v1 & v8) + (v13 & v2) + (v13 & v5) + (v13 & v7) + (v2 & v14) + (v2 & v5) + (v2 & v6) + (v14 & v6) + (v14 & v8) + (v3 & v15) + (v3 & v10) + (v4 & v16) + (v4 & v11) + (v5 & v15) + (v5 & v9) + (v6 & v9) + (v6 & v16) + (v7 & v11) + (v7 & v17) + (v8 & v10) + (v8 & v17) + (v15 & v9) + (v15 & v10) + (v9 & v16) + (v16 & v11) + (v10 & v17) + (v11 & v17);
  const unsigned lo = ((unsigned)v0 << 0) | ((unsigned)v1 << 1) | ((unsigned)v2 << 2) | ((unsigned)v3 << 3) | ((unsigned)v4 << 4) | ((unsigned)v5 << 5) | ((unsigned)v6 << 6) | ((unsigned)v7 << 7) | ((unsigned)v8 << 8) | ((unsigned)v9 << 9) | ((unsigned)v10 << 10) | ((unsigned)v11 << 11) | ((unsigned)v12 << 12) | ((unsigned)v13 << 13) | ((unsigned)v14 << 14) | ((unsigned)v15 << 15) | ((unsigned)v16 << 16) | ((unsigned)v17 << 17) | ((unsigned)v18 << 18) | ((unsigned)v19 << 19) | ((unsigned)v20 << 20) | ((unsigned)v21 << 21) | ((unsigned)v22 << 22) | ((unsigned)v23 << 23) | ((unsigned)v24 << 24) | ((unsigned)v25 << 25) | ((unsigned)v26 << 26) | ((unsigned)v27 << 27) | ((unsigned)v28 << 28) | ((unsigned)v29 << 29) | ((unsigned)v30 << 30) | ((unsigned)v31 << 31);
  const unsigned hi = ((unsigned)v32 << 0) | ((unsigned)v33 << 1) | ((unsigned)v34 << 2) | ((unsigned)v35 << 3) | ((unsigned)v36 << 4) | ((unsigned)v37 << 5) | ((unsigned)v38 << 6) | ((unsigned)v39 << 7) | ((unsigned)v40 << 8) | ((unsigned)v41 << 9);
  env = ((unsigned long long)hi << 32) | lo;
}

// owned[g] = number of clusters of orbit g anchored at this site (its
// lexicographically smallest point) whose other sites are all 1
template <int P>
__device__ __forceinline__ void owned_counts(const int8_t *__restrict__ c,
                                             int (&n)[N_ORBITS]) {
  const int v1 = c[(-1) + P * (0) + P * P * (1)];
  const int v2 = c[(-1) + P * (1) + P * P * (0)];
  const int v4 = c[(0) + P * (-1) + P * P * (1)];
  const int v6 = c[(0) + P * (0) + P * P * (1)];
  const int v8 = c[(0) + P * (1) + P * P * (0)];
  const int v11 = c[(1) + P * (0) + P * P * (0)];
  const int v14 = c[(-1) + P * (1) + P * P * (1)];
  const int v16 = c[(1) + P * (-1) + P * P * (1)];
  const int v17 = c[(1) + P * (1) + P * P * (-1)];
  const int v18 = c[(-2) + P * (0) + P * P * (1)];
  const int v19 = c[(-2) + P * (1) + P * P * (0)];
  const int v20 = c[(-2) + P * (1) + P * P * (1)];
  const int v22 = c[(-1) + P * (-1) + P * P * (2)];
  const int v24 = c[(-1) + P * (0) + P * P * (2)];
  const int v25 = c[(-1) + P * (2) + P * P * (-1)];
  const int v26 = c[(-1) + P * (2) + P * P * (0)];
  const int v29 = c[(0) + P * (-1) + P * P * (2)];
  const int v31 = c[(0) + P * (1) + P * P * (1)];
  const int v32 = c[(0) + P * (2) + P * P * (-1)];
  const int v36 = c[(1) + P * (0) + P * P * (1)];
  const int v38 = c[(1) + P * (1) + P * P * (0)];
  n[0] = 1;
  n[1] = v1 + v2 + v4 + v6 + v8 + v11;
  n[2] = v14 + v16 + v17;
  n[3] = v18 + v19 + v20 + v22 + v24 + v25 + v26 + v29 + v31 + v32 + v36 + v38;
  n[4] = (v1 & v2) + (v1 & v4) + (v1 & v6) + (v2 & v8) + (v4 & v6) + (v6 & v8) + (v6 & v11) + (v8 & v11);
  n[5] = (v1 & v14) + (v1 & v8) + (v2 & v14) + (v2 & v6) + (v14 & v6) + (v14 & v8) + (v4 & v16) + (v4 & v11) + (v6 & v16) + (v8 & v17) + (v16 & v11) + (v11 & v17);
}

}  // namespace gen_fcc
}  // namespace cem
