// Drop-in check of the reference-side binding (banjo_gb300/adapter).
//
// A reference program, unchanged: it builds a box lattice through the
// reference's own generator, schedule and state builders, then asks the
// reference's CUDA factory for a backend. With the binding linked in place of
// the reference's CUDA stub, the factory is the GB300 library. Without a device
// the factory throws std::runtime_error, as the stub's contract says; with one,
// the GB300 backend is run against CpuLatticeBackend<float> and must agree bit
// for bit (the reference's own CUDA test, tests/fast_lattice_tests.cpp:480-524).
// Prints one line per check and exits non-zero on a mismatch.
#include "fastlattice/FastLattice.hpp"
#include "fastlattice/LatticeSchedule.hpp"
#include "matter/BoxLattice.hpp"
#include "material/MaterialCompiler.hpp"

#include <cstdio>
#include <memory>
#include <stdexcept>

using namespace banjo;
using namespace banjo::fastlattice;

int main() {
    MaterialDefinition glass{};
    glass.model = MaterialModel::BrittleBond;
    glass.density_kg_m3 = 2500;
    glass.young_modulus_pa = 70e9;
    glass.poisson_ratio = 0.22;
    glass.tensile_strength_pa = 45e6;
    const double cell = 0.02;
    const auto compiled = withStrengthDerivedFailure(compileElasticLatticeReference(glass, cell, 2), glass);
    BoxLatticeLayout layout{};
    const auto asset = std::make_unique<LatticeAsset>(generateBoxTileLattice({{0.12, 0.04, 0.16}, cell, 2}, compiled, &layout));
    ActiveMatter matter;
    matter.asset = asset.get();
    matter.material = compiled;
    for (const auto &node : asset->nodes) {
        matter.nodes.push_back({node.local_position_m, node.local_position_m, {0.0, -3.0, 0.0},
                                node.represented_volume_m3 * compiled.density_kg_m3, {}});
        matter.reference_positions_world_m.push_back(node.local_position_m);
    }
    matter.bonds.resize(asset->bonds.size());
    const LatticeSchedule schedule = buildLatticeSchedule(*asset, boxLatticeSlabs(layout, 2, 2));
    LatticeState state = buildLatticeState(matter, schedule, Vec3{});
    StepSettings<double> settings{};
    settings.dt = 1.0 / 2400.0;
    settings.gravity = {0.0, -9.81, 0.0};
    settings.constraint_iterations = 4;
    SphereState<double> sphere{};

    std::printf("cudaLatticeAvailable=%d description=\"%s\" sms=%u\n", cudaLatticeAvailable() ? 1 : 0,
                cudaLatticeDescription().c_str(), cudaLatticeMultiprocessorCount());
    if (!cudaLatticeAvailable()) {
        try {
            (void)makeCudaLatticeBackend(schedule, Precision::Float, 256);
            std::printf("FAIL: the factory returned a backend without a device\n");
            return 1;
        } catch (const std::runtime_error &e) {
            std::printf("PASS: no device, factory threw runtime_error: %s\n", e.what());
            return 0;
        }
    }
    auto gpu = makeCudaLatticeBackend(schedule, Precision::Float, 256);
    auto cpu = makeCpuLatticeBackend(schedule, Precision::Float);
    gpu->upload(state, settings, sphere);
    cpu->upload(state, settings, sphere);
    RunControl control{};
    control.max_steps = 200;
    const RunStatus gs = gpu->run(control), cs = cpu->run(control);
    LatticeState a = state, b = state;
    SphereState<double> sa{}, sb{};
    gpu->download(a, sa);
    cpu->download(b, sb);
    const bool same = a.u == b.u && a.v == b.v && a.alive == b.alive && a.damage == b.damage &&
                      gs.broken_bonds == cs.broken_bonds && gs.total_steps == cs.total_steps;
    std::printf("%s: %s vs %s, %u broken, %llu steps\n", same ? "PASS" : "FAIL", gpu->name().c_str(),
                cpu->name().c_str(), gs.broken_bonds, static_cast<unsigned long long>(gs.total_steps));
    return same ? 0 : 1;
}
