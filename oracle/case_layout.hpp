// Fixed packing of the step settings and sphere records of a lattice case file.
//
// Test infrastructure only: the reference harness, the CPU restatement and the
// Python test/bench side all pack StepSettings<double> and SphereState<double>
// (src/fastlattice/LatticePhysics.hpp:144-158, 248-284) into these flat f64
// arrays in this one order.
#pragma once

namespace lsio {

enum SettingsSlot : int {
    kDt = 0,
    kGravity = 1,            // 3
    kIterations = 4,
    kDampingFraction = 5,
    kSphereEnabled = 6,
    kDirectArithmetic = 7,
    kPlasticYield = 8,
    kPlasticHardening = 9,
    kPlateHalfThickness = 10,
    kContact = 11,           // 7: static, dynamic, restitution, threshold, node radius, margin, slack
    kPlaneCount = 18,
    kPlanes = 19,            // 2 x kPlaneWidth
    // 9: mode, radius, skin, margin, restitution, restitution speed threshold,
    // static friction, dynamic friction, bucket mask. A record that ends here
    // (kNodeContact wide) has node-to-node contact off.
    kNodeContact = 19 + 2 * 34,
    // StepSettings::audit_energy. A record that ends before it has the audit off.
    kAuditEnergy = kNodeContact + 9,
    kSettingsWidth = kAuditEnergy + 1,
};

enum PlaneSlot : int {
    kPlanePoint = 0,         // 3
    kPlaneNormal = 3,        // 3
    kPlaneTangent = 6,       // 3
    kPlaneBitangent = 9,     // 3
    kPlaneRestitution = 12,
    kPlaneStatic = 13,
    kPlaneDynamic = 14,
    kPlaneNodeRadius = 15,
    kPlaneReachCapped = 16,
    kPlaneFootprintCount = 17,
    kPlaneFootprints = 18,   // 4 x (center_t, center_b, half_t, half_b)
    kPlaneWidth = 34,
};

// center 3, velocity 3, angular velocity 3, radius, mass, inertia
constexpr int kSphereWidth = 12;

// External wrenches (FastLattice.hpp:153-157) in a case: `wrench_names` (each
// name followed by a zero byte), `wrench_node_count` and the concatenated
// `wrench_nodes`, `wrench_vectors` (point, force, torque per wrench) and
// `wrench_substeps`. A run's source ledgers come back as `source_names` and
// `source_ledgers`: steps, elapsed, requested impulse 3, impulse 3, requested
// angular impulse 3, angular impulse 3, work per source, in status order.
constexpr int kWrenchWidth = 9;
constexpr int kSourceLedgerWidth = 15;

// Status packing shared by every runner that reports a RunStatus.
enum StatusU64Slot : int {
    kTotalSteps = 0,
    kFirstFailureStep,
    kLastFailureStep,
    kFailureRounds,
    kBrokenBonds,
    kLastEnergyGainStep,
    kLastDamageGainStep,
    kExitReason,
    kRankDeficientNodes,
    kImpulseContacts,
    kCandidateOverflow,
    kBallSupportEvents,
    kLaunches,
    kNodeContacts,           // node-to-node contact (NodeContactAccumulators)
    kNodePairTests,
    kNodeRebuilds,
    kNodePairsListed,
    kNodePairOverflow,
    kEnergyAudited,          // RunStatus::energy_audited
    kStatusU64Width,
};

enum StatusF64Slot : int {
    kRemovedEnergy = 0,
    kMaxDamage,
    kPlasticWork,
    kMaxTensile,
    kMaxCompressive,
    kMaxShear,
    kMaxPlasticStretch,
    kImpulseX,
    kImpulseY,
    kImpulseZ,
    kContactDissipated,
    kMaxPenetration,
    kMaxCorrection,
    kMaxCenterShift,
    kExternalWork,
    kExternalImpulseX,
    kExternalImpulseY,
    kExternalImpulseZ,
    kExternalSteps,
    kWallSeconds,
    kNodeDissipated,         // node-to-node contact (NodeContactAccumulators)
    kNodeMaxOverlap,
    kNodeMaxCorrection,
    kNodeMomentumX,
    kNodeMomentumY,
    kNodeMomentumZ,
    kDampingDissipated,      // the energy audit (StepSettings::audit_energy)
    kStrikerDissipated,
    kStatusF64Width,
};

} // namespace lsio
