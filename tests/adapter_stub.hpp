// A recording stand-in for the lattice library, for the adapter's field test.
//
// tests/adapter_stub.cpp implements the entry points of include/gbl.h that the
// reference-side binding (banjo_gb300/adapter/Gb300LatticeBackend.cpp) calls.
// Every struct and array the binding passes in is copied into the record below;
// everything the binding reads back (RunStatus, downloaded state, sources,
// first-failure bonds, frames) is filled with distinct values the driver
// (tests/adapter_stub_driver.cpp) knows, so each field's path through the
// binding can be checked on its own, with no device.
#pragma once

#include "gbl.h"

#include <cstdint>
#include <string>
#include <vector>

namespace stub {

struct Record {
    // gbl_create
    gbl_schedule_view schedule{};
    std::vector<std::uint32_t> node_block_begin, bond_order, bond_schedule_index, bond_block_begin, range_begin,
        range_end;
    std::vector<std::uint8_t> bond_color;
    int precision{-1};
    unsigned threads_per_block{};
    // gbl_upload
    gbl_state_view state{};
    std::vector<double> x0, u, u_prev, v, inv_mass, mass, nbr_rest, nbr_weight, rest_edge, rest_length,
        rest_length_sq_minus, weight, compliance, threshold, damage, prev_tensile, prev_compressive, prev_shear,
        plastic_extension, plastic_strain;
    std::vector<std::uint32_t> adj_offsets, adj_bonds, nbr_bond, nbr_other, bond_slot_a, bond_slot_b, bond_a, bond_b;
    std::vector<std::uint8_t> nbr_alive, alive, failure_mode;
    gbl_step_settings settings{};
    gbl_sphere sphere{};
    // gbl_set_external_forces / gbl_set_external_wrenches
    std::vector<double> forces;
    std::uint64_t force_count{}, force_substeps{};
    struct Wrench {
        std::string source;
        std::vector<std::uint32_t> nodes;
        double point[3], force[3], torque[3];
    };
    std::vector<Wrench> wrenches;
    std::uint64_t wrench_substeps{};
    // gbl_run
    gbl_run_control control{};
    int runs{};
    int destroyed{};
};

Record &record();

// What the stub hands back, as the driver expects it.
gbl_run_status statusPattern();
gbl_load_ledger sourceLedger(unsigned k);
const char *sourceName(unsigned k);
constexpr unsigned kSources = 2;
gbl_sphere downloadedSphere();
double downloaded(unsigned array, std::size_t i); // value of element i of download array `array`
constexpr std::uint32_t kFirstFailure[3] = {5, 3, 9};
constexpr unsigned kFrames = 2;
float frameValue(unsigned frame, unsigned array, std::size_t i);
gbl_sphere frameSphere(unsigned frame);
constexpr const char *kName = "stub-gb300";
constexpr const char *kDescription = "stub device, no GPU";
constexpr unsigned kMultiprocessors = 152;

} // namespace stub
