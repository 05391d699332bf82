// devmech.h - the mechanism as the GPU reads it: one device allocation holding flat
// arrays, addressed through the pointers below.  Built on the host from a Mechanism
// (mechanism.h) by packDevMech() in capi.cu.
#pragma once
#include <cstdint>

#ifndef __CUDACC__
struct int4 { int x, y, z, w; };
#else
#include <cuda_runtime.h>
#endif

namespace gbchem {

// four doubles, 32-byte aligned (loaded as two 16-byte vector loads)
struct alignas(32) D4 { double x, y, z, w; };

constexpr int kMaxSpecies = 255;   // limits of the GPU path (checked at load time)
constexpr int kMaxN = kMaxSpecies + 1;   // integrated components: T and the species
constexpr int kNasaStride = 16;    // Tmid, low[7], high[7], pad

// rinfo.x bit fields
constexpr int kKindMask = 0x7;      // RateKind
constexpr int kRevBit = 1 << 3;     // reversible
constexpr int kRBucketShift = 4;    // reactant StoichBucket (3 bits)
constexpr int kPBucketShift = 7;    // product StoichBucket (3 bits)
constexpr int kDnIntBit = 1 << 10;  // dn is an integer in [-3, 3]
constexpr int kNoExpBit = 1 << 11;  // b = 0 and Ea = 0: k = A

struct DevMech {
    int K, R, N, NF, NTB, nnz;
    double Pref, Rgas;
    // species [K]
    const double* mw;
    const double* rmw;
    const double* nasa;          // [K][kNasaStride]
    // reactions [R]
    const int4* rinfo;           // x flags, y third-body index (-1), z falloff index (-1), w unused
    const D4* rarr;         // A, b, Ea/R, dn
    const int4* rk;              // reactant species repeated by coefficient (x,y,z; -1 unused), w = count
    const int4* pk;              // product species, same form
    const int* sidePtr;          // [2R+1] general side lists (used by CN buckets): side 2i reactants, 2i+1 products
    const int* sideK;
    const double* sideNu;
    const double* sideOrd;
    const int* rsPtr;            // [R+1] species of reaction i with net stoichiometric coefficient
    const int* rsK;
    const double* rsNu;
    // falloff [NF]
    const D4* fo1;          // A0, b0, Ea0/R, Troe a
    const D4* fo2;          // 1/T3, 1/T1, T2, isTroe
    // third bodies [NTB]
    const int* tbRxn;
    const double* tbDef;
    const int* tbMA;
    const int* tbPtr;            // [NTB+1]
    const int* tbK;
    const double* tbE;           // efficiency - default
    // wdot gather: species k -> (reaction, net coefficient)
    const int* spPtr;            // [K+1]
    const int* spRxn;
    const double* spNu;
    // the same entries cut into tasks of bounded length for a balanced warp gather:
    // task t sums entries [taskPtr[t], taskPtr[t+1]) of one species; lane l runs tasks
    // laneTasks[laneTaskPtr[l] .. laneTaskPtr[l+1]); species k adds the partial sums of
    // tasks spTasks[spTaskPtr[k] .. spTaskPtr[k+1]) in order
    int NT;
    const int* taskPtr;          // [NT+1] into spRxn / spNu
    const int* laneTaskPtr;      // [33]
    const int* laneTasks;
    const int* spTaskPtr;        // [K+1]
    const int* spTasks;
    // d(wdot)/dc columns: column j -> (reaction, efficiency - default of j or 0)
    const int* colPtr;           // [K+1]
    const int* colRxn;
    const double* colE;
    const int* laneColPtr;       // [33] columns assigned to each lane (balanced by work)
    const int* laneCols;
    // dense default-efficiency part: species k -> (third-body index, S_net[k][i] * default)
    const int* gsPtr;            // [K+1]
    const int* gsTb;
    const double* gsCoef;
    // output pattern of d(wdot)/dc (CSC): jcPtr[K+1], jrIdx[nnz], jpCol[nnz] (column of each slot)
    const int* jcPtr;
    const int* jrIdx;
    const int* jpCol;
};

}  // namespace gbchem
