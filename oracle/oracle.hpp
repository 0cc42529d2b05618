// CPU restatement of the reference's bonded-lattice XPBD fracture substep.
//
// TEST INFRASTRUCTURE ONLY. This library is the checker the GPU path is proven
// against; nothing in the product links, loads or calls it. Only tests, the
// smoke check and the CPU-baseline leg of the benchmark may use it.
//
// It restates, in its own code, the reference's CPU float/double lane:
//   src/fastlattice/LatticeSchedule.cpp:71-155   greedy colouring, slab split
//   src/fastlattice/FastLattice.cpp:47-169       canonical state build
//   src/fastlattice/LatticeWorking.hpp:53-124    working copy
//   src/fastlattice/LatticePhysics.hpp           element physics
//   src/fastlattice/CpuLatticeBackend.cpp:255-488 run / advance / finishStep
//   src/fastlattice/ExternalLoads.hpp:28-148     external force kick and ledger
// Its outputs are pinned bit for bit to the reference itself (oracle/_ref,
// built from the reference's own sources) by the golden fixtures under
// tests/golden and by tests/test_oracle_pin.py.
//
// A case is a bag of named arrays (oracle/lsio.hpp); the run reads the inputs
// named in oracle/case_layout.hpp and writes the same outputs the reference
// harness writes.
#pragma once

#include <cstdint>

#ifdef __cplusplus
extern "C" {
#endif

void *oracle_case_new(void);
void oracle_case_free(void *c);
int oracle_case_put(void *c, const char *name, char type, std::uint64_t count, const void *data);
// Element count of a named array, -1 when the case has none.
long long oracle_case_count(void *c, const char *name);
char oracle_case_type(void *c, const char *name);
int oracle_case_get(void *c, const char *name, void *dst, std::uint64_t bytes);
int oracle_case_read(void *c, const char *path);
int oracle_case_write(void *c, const char *path);
// precision: 0 float (displacement arithmetic), 1 double (direct arithmetic).
// threads: 1 for the serial lane, more for the colour-parallel lane (bit
// identical). per_substep: also record the substep at which each bond broke.
int oracle_run(void *in_case, void *out_case, int precision, int threads, int per_substep);
const char *oracle_last_error(void);

#ifdef __cplusplus
}
#endif
