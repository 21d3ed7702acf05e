// fau_faunus.hpp -- Faunus plugin classes over the C ABI of libfau_gpu (include/fau_gpu.h).
//
// What a maintainer adds to the reference to run its Metropolis energy hot path on the GPU:
//
//   DeviceSystem         one resident system (Space + the Nonbonded, Ewald and self-energy terms),
//                        shared by the accepted and the trial Hamiltonian of a
//                        MetropolisMonteCarlo (src/montecarlo.cpp:100-111): the accepted state
//                        lives on the device, one trial move at a time is pending on it
//                        (fau_energy_change / fau_commit_pending).
//   NonbondedEwaldGPU    an Energy::EnergyTerm (src/externalpotential.h:17-38) standing for the
//                        ParticleSelfEnergy, Nonbonded and Ewald terms together; one instance in
//                        each of the two Hamiltonians.
//   ReferenceStreamMove  a move::Move (src/move.h:38-76) drawing MoveCollection::sample and the
//                        transrot / moltransrot / volume proposals from the reference's mt19937
//                        streams (fau_movegen), which hands each proposal to the DeviceSystem.
//
// performMove (src/montecarlo.cpp:139-187) then runs unchanged:
//   move.move(change)                        -> the proposal is pending on the device
//   trial.updateState(change)                -> the trial is evaluated once (fau_energy_change)
//   new = trial.energy(change)               -> the trial state's energy
//   old = accepted.energy(change)            -> the accepted state's energy
//   getEnergyChange(new, old), metropolisCriterion
//   accepted.sync(trial) | trial.sync(accepted) -> fau_commit_pending(1 | 0)
//
// Energies returned are the states' totals (self + nonbonded + Ewald, the Change::everything
// form): new - old is the device's energy change to the rounding of the total, and a state with
// an overlap or a NaN returns +inf or the change's own infinity, so getEnergyChange's policy and
// Hamiltonian::energy's `maxenergy` stop act on them as on the reference terms' values.
//
// In the reference tree, include "space.h", "energy.h" and "move.h" instead of
// faunus_interfaces.hpp.
#pragma once

#include "fau_gpu.h"
#include "faunus_interfaces.hpp"

#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace faunus_gpu {

inline void check(int rc, const char* what)
{
    if (rc != FAU_OK)
        throw std::runtime_error(std::string(what) + ": " + fau_strerror(rc) + " (" + fau_last_error() + ")");
}

class DeviceSystem {
  public:
    DeviceSystem(fau_ctx* ctx, const fau_sys_desc& desc)
    {
        check(fau_sys_create(ctx, &desc, &sys_), "fau_sys_create");
        check(fau_refresh_energy(sys_, &energy_), "fau_refresh_energy");
    }
    ~DeviceSystem()
    {
        if (sys_) fau_sys_destroy(sys_);
    }
    DeviceSystem(const DeviceSystem&) = delete;
    DeviceSystem& operator=(const DeviceSystem&) = delete;

    fau_sys* handle() const { return sys_; }

    // the move's proposal (ReferenceStreamMove::_move)
    void propose(const fau_proposal& p)
    {
        proposal_ = p;
        pending_proposal_ = true;
        evaluated_ = false;
    }
    // Hamiltonian::updateState of the trial state: the pending trial is evaluated once
    void evaluate()
    {
        if (!pending_proposal_ || evaluated_) return;
        check(fau_energy_change(sys_, &proposal_, &trial_), "fau_energy_change");
        evaluated_ = true;
    }
    // the accepted state's total energy (+inf when it holds an overlap)
    double accepted_energy() const { return evaluated_ && trial_.old_inf ? INFINITY : energy_; }
    // the trial state's total energy: the accepted one plus the change, or the change's infinity
    double trial_energy() const
    {
        if (!evaluated_) return energy_;
        if (trial_.new_inf) return INFINITY;
        return std::isfinite(trial_.du) ? energy_ + trial_.du : trial_.du;
    }
    const fau_trial_result& trial() const { return trial_; }

    // State::sync: 1 = trial -> accepted (accept), 0 = accepted -> trial (reject)
    void commit(bool accept)
    {
        if (!evaluated_) return;
        check(fau_commit_pending(sys_, accept ? 1 : 0), "fau_commit_pending");
        if (accept) {
            if (std::isfinite(trial_.du) && std::isfinite(energy_)) energy_ += trial_.du;
            else check(fau_refresh_energy(sys_, &energy_), "fau_refresh_energy");
        }
        pending_proposal_ = evaluated_ = false;
    }

  private:
    fau_sys* sys_ = nullptr;
    fau_proposal proposal_{};
    fau_trial_result trial_{};
    bool pending_proposal_ = false, evaluated_ = false;
    double energy_ = 0.0;
};

class NonbondedEwaldGPU : public Faunus::Energy::EnergyTerm {
  public:
    explicit NonbondedEwaldGPU(std::shared_ptr<DeviceSystem> dev) : dev_(std::move(dev))
    {
        name = "nonbonded+ewald+self (gpu)";
    }
    double energy(const Faunus::Change& change) override
    {
        if (!change) return 0.0;
        if (state == MonteCarloState::TRIAL) {
            dev_->evaluate();
            return dev_->trial_energy();
        }
        return dev_->accepted_energy();
    }
    void updateState(const Faunus::Change& change) override
    {
        if (state == MonteCarloState::TRIAL && change) dev_->evaluate();
    }
    // accepted.sync(trial) after an accepted move; trial.sync(accepted) after a rejected one
    void sync(Faunus::Energy::EnergyTerm* /*other*/, const Faunus::Change& change) override
    {
        if (change) dev_->commit(state == MonteCarloState::ACCEPTED);
    }

  private:
    std::shared_ptr<DeviceSystem> dev_;
};

class ReferenceStreamMove : public Faunus::move::Move {
  public:
    // `space` is the descriptor the system was made from (its group layout); moves and seeds as
    // fau_movegen_create takes them
    ReferenceStreamMove(std::shared_ptr<DeviceSystem> dev, const fau_sys_desc& space, const fau_move_desc* moves,
                        int n_moves, uint32_t slump_seed, uint32_t random_seed, bool default_seeds)
        : dev_(std::move(dev)), group_begin_(space.group_begin, space.group_begin + space.n_groups + 1)
    {
        check(fau_movegen_create(&space, moves, n_moves, slump_seed, random_seed, default_seeds ? 1 : 0, &gen_),
              "fau_movegen_create");
    }
    ~ReferenceStreamMove() override
    {
        if (gen_) fau_movegen_destroy(gen_);
    }
    ReferenceStreamMove(const ReferenceStreamMove&) = delete;
    ReferenceStreamMove& operator=(const ReferenceStreamMove&) = delete;

    // the Metropolis uniform the reference draws from Move::slump after this move
    double uniform() const { return last_.u; }
    const fau_proposal& last() const { return last_; }

  private:
    void _move(Faunus::Change& change) override
    {
        check(fau_movegen_generate(gen_, &last_, 1), "fau_movegen_generate");
        if (last_.kind == FAU_MOVE_NONE) return; // empty Change
        if (last_.kind == FAU_MOVE_VOLUME)
            throw std::runtime_error("volume moves go through fau_volume_move, not the two-phase trial");
        dev_->propose(last_);
        Faunus::Change::GroupChange g;
        if (last_.kind == FAU_MOVE_ATOMIC) {
            int grp = 0;
            while (grp + 1 < (int)group_begin_.size() - 1 && group_begin_[grp + 1] <= last_.index) grp++;
            g.group_index = (Faunus::Change::index_type)grp;
            g.internal = true;
            g.relative_atom_indices.push_back((Faunus::Change::index_type)(last_.index - group_begin_[grp]));
        }
        else {
            g.group_index = (Faunus::Change::index_type)last_.index;
            g.all = true;
        }
        change.groups.push_back(std::move(g));
    }

    std::shared_ptr<DeviceSystem> dev_;
    std::vector<int> group_begin_;
    fau_movegen* gen_ = nullptr;
    fau_proposal last_{};
};

} // namespace faunus_gpu
