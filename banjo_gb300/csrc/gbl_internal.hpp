// Internal host-side types shared by the C ABI translation units.
#pragma once

#include "gbl.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace gbl {

constexpr std::uint64_t kNodeLimit = 1ULL << 30; // node indices keep two flag bits free

// Exceptions carry the gbl_result the C ABI returns for them; the names follow
// the reference's exception types (FastLattice.hpp:263-358).
struct Error : std::runtime_error {
    gbl_result code;
    Error(gbl_result c, const std::string &m) : std::runtime_error(m), code(c) {}
};
[[noreturn]] inline void invalid(const std::string &m) { throw Error(GBL_INVALID_ARGUMENT, m); }
[[noreturn]] inline void runtime(const std::string &m) { throw Error(GBL_RUNTIME_ERROR, m); }
[[noreturn]] inline void overflow(const std::string &m) { throw Error(GBL_OVERFLOW_ERROR, m); }
[[noreturn]] inline void logic(const std::string &m) { throw Error(GBL_LOGIC_ERROR, m); }

void setLastError(const std::string &m);

template <class F> gbl_result guard(F &&f) noexcept {
    try {
        f();
        return GBL_OK;
    } catch (const Error &e) {
        setLastError(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        setLastError("host allocation failed");
        return GBL_RUNTIME_ERROR;
    } catch (const std::exception &e) {
        setLastError(e.what());
        return GBL_RUNTIME_ERROR;
    }
}

// LatticeSchedule with owned arrays (LatticeSchedule.hpp:28-44).
struct Schedule {
    std::uint32_t node_count{}, bond_count{}, block_count{1}, color_count{}, boundary_bond_count{};
    std::vector<std::uint32_t> node_block_begin, bond_order, bond_schedule_index, bond_block_begin, range_begin, range_end;
    std::vector<std::uint8_t> bond_color;

    static Schedule fromView(const gbl_schedule_view &v);
    [[nodiscard]] gbl_schedule_view view() const;
    [[nodiscard]] std::size_t rangeKey(std::uint32_t block, std::uint32_t boundary, std::uint32_t color) const {
        const std::uint32_t c = color_count > 0 ? color_count : 1;
        return (static_cast<std::size_t>(block) * 2 + boundary) * c + color;
    }
};

Schedule buildSchedule(std::uint32_t node_count, std::uint32_t bond_count, const std::uint32_t *a, const std::uint32_t *b,
                       const std::uint32_t *node_block_begin, std::uint32_t block_count);

// LatticeState with owned arrays (FastLattice.hpp:37-55).
struct State {
    double origin[3]{};
    std::uint32_t node_count{}, bond_count{}, max_degree{};
    std::vector<double> x0, u, u_prev, v, inv_mass, mass;
    std::vector<std::uint32_t> adj_offsets, adj_bonds, nbr_bond, nbr_other;
    std::vector<double> nbr_rest, nbr_weight;
    std::vector<std::uint8_t> nbr_alive;
    std::vector<std::uint32_t> bond_slot_a, bond_slot_b, bond_a, bond_b;
    std::vector<double> rest_edge, rest_length, rest_length_sq_minus, weight, compliance, threshold;
    std::vector<std::uint8_t> alive, failure_mode;
    std::vector<double> damage, prev_tensile, prev_compressive, prev_shear, plastic_extension, plastic_strain;

    [[nodiscard]] gbl_state_view view();
};

State buildState(const gbl_matter_view &m, const Schedule &s, const double origin[3]);

// The unique ID of the current CUDA context (cuCtxGetId), or 0 when none is
// current or the driver cannot say. A context created after a device reset
// has a new ID, so device pointers and pinned host buffers cached against an
// ID are known to be stale once it changes.
unsigned long long currentContextId();

} // namespace gbl

struct gbl_schedule {
    gbl::Schedule s;
};
struct gbl_state {
    gbl::State s;
};
