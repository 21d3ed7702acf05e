// faunus_interfaces.hpp -- the parts of Faunus's plugin surface the GPU adaptor is written
// against, declared with the reference's names and signatures so that the adaptor compiles
// and is tested here without the reference tree.  In the reference tree these declarations
// come from its own headers instead:
//
//   Faunus::Change                      src/space.h:29-75
//   Faunus::Energy::EnergyTerm          src/externalpotential.h:17-38
//   Faunus::Energy::Hamiltonian         src/energy.h (energy(), updateState(), sync();
//                                       src/energy.cpp:1227-1268, with `maxenergy`)
//   Faunus::move::Move                  src/move.h:38-76
//
// Only what the adaptor and its test use is here; bodies are the minimum those members need.
#pragma once

#include <cmath>
#include <cstddef>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

namespace Faunus {

// What a move touched: the groups and, within each, the changed atoms (src/space.h:29-75).
struct Change {
    using index_type = std::size_t;
    bool everything = false;
    bool volume_change = false;
    bool matter_change = false;
    bool moved_to_moved_interactions = true;
    bool disable_translational_entropy = false;
    struct GroupChange {
        index_type group_index = 0;
        bool dNatomic = false;
        bool dNswap = false;
        bool internal = false;
        bool all = false;
        std::vector<index_type> relative_atom_indices;
    };
    std::vector<GroupChange> groups;

    void clear() { *this = Change(); }
    [[nodiscard]] bool empty() const { return !everything && !volume_change && !matter_change && groups.empty(); }
    explicit operator bool() const { return !empty(); }
};

namespace Energy {

// An energy term of a Hamiltonian (src/externalpotential.h:17-38).
class EnergyTerm {
  public:
    enum class MonteCarloState { ACCEPTED, TRIAL, NONE };
    MonteCarloState state = MonteCarloState::NONE;
    std::string name;
    virtual double energy(const Change& change) = 0;
    virtual void sync(EnergyTerm* /*other_energy*/, const Change& /*change*/) {}
    virtual void init() {}
    virtual void updateState(const Change& /*change*/) {}
    virtual ~EnergyTerm() = default;
};

// The sum of the terms in order, stopping at a term whose energy is >= maximum_allowed_energy or
// NaN (Hamiltonian::energy, src/energy.cpp:1227-1241; `maxenergy` in the input, default +inf).
class Hamiltonian : public EnergyTerm {
  public:
    std::vector<std::shared_ptr<EnergyTerm>> energy_terms;
    double maximum_allowed_energy = INFINITY;
    std::vector<double> latest_energies;

    double energy(const Change& change) override
    {
        latest_energies.clear();
        for (auto& term : energy_terms) {
            term->state = state;
            const double e = term->energy(change);
            latest_energies.push_back(e);
            if (e >= maximum_allowed_energy || std::isnan(e)) break;
        }
        return std::accumulate(latest_energies.begin(), latest_energies.end(), 0.0);
    }
    void updateState(const Change& change) override
    {
        for (auto& term : energy_terms) term->updateState(change);
    }
    void sync(EnergyTerm* other, const Change& change) override
    {
        auto* h = dynamic_cast<Hamiltonian*>(other);
        for (std::size_t i = 0; i < energy_terms.size(); i++) energy_terms[i]->sync(h->energy_terms[i].get(), change);
    }
    void init() override
    {
        for (auto& term : energy_terms) term->init();
    }
};

} // namespace Energy

namespace move {

// A Monte Carlo move (src/move.h:38-76): _move fills the Change; accept / reject follow the
// Metropolis decision; bias is the extra energy a move adds to it.
class Move {
  public:
    void move(Change& change)
    {
        number_of_attempted_moves++;
        _move(change);
    }
    void accept(Change& change)
    {
        number_of_accepted_moves++;
        _accept(change);
    }
    void reject(Change& change)
    {
        number_of_rejected_moves++;
        _reject(change);
    }
    virtual double bias(Change& /*change*/, double /*old_energy*/, double /*new_energy*/) { return 0.0; }
    virtual ~Move() = default;
    unsigned long attempted() const { return number_of_attempted_moves; }
    unsigned long accepted() const { return number_of_accepted_moves; }

  private:
    virtual void _move(Change& change) = 0;
    virtual void _accept(Change& /*change*/) {}
    virtual void _reject(Change& /*change*/) {}
    unsigned long number_of_accepted_moves = 0;
    unsigned long number_of_rejected_moves = 0;

  protected:
    unsigned long number_of_attempted_moves = 0;
};

} // namespace move
} // namespace Faunus
