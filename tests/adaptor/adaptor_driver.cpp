// adaptor_driver.cpp -- a MetropolisMonteCarlo::performMove loop (reference
// src/montecarlo.cpp:139-187, getEnergyChange :193-209, metropolisCriterion :17-34) written
// against the Faunus plugin interfaces, with the GPU adaptor classes of
// faunus_gb300/adaptor/fau_faunus.hpp as its energy term and move.  Built as a shared library
// by tests/test_adaptor.py and called through ctypes; the test compares what it returns with
// the FP64 oracle replaying the same reference-stream proposals.
#include "fau_faunus.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <exception>
#include <limits>

namespace {

// getEnergyChange (src/montecarlo.cpp:193-209)
double energy_change(double new_energy, double old_energy)
{
    if (std::isnan(old_energy) && !std::isnan(new_energy)) return -std::numeric_limits<double>::infinity();
    if (std::isnan(new_energy)) return std::numeric_limits<double>::infinity();
    if (new_energy > 0.0 && std::isinf(new_energy)) return std::numeric_limits<double>::infinity();
    const double du = new_energy - old_energy;
    return std::isnan(du) ? 0.0 : du;
}

// metropolisCriterion (src/montecarlo.cpp:17-34) on the uniform the move drew
bool metropolis(double du, double u)
{
    if (std::isinf(du) && du < 0.0) return true;
    if (-du > 709.782712893384) return true;
    return u <= std::exp(-du);
}

} // namespace

extern "C" int adaptor_run(const fau_sys_desc* desc, const fau_move_desc* moves, int n_moves, uint32_t slump_seed,
                           uint32_t random_seed, double maxenergy, int n, uint8_t* acc_out, double* du_out,
                           double* energy_out, char* err, int errlen)
{
    using Faunus::Change;
    using Faunus::Energy::EnergyTerm;
    try {
        fau_ctx* ctx = nullptr;
        faunus_gpu::check(fau_ctx_create(0, 0, &ctx), "fau_ctx_create");
        {
            auto dev = std::make_shared<faunus_gpu::DeviceSystem>(ctx, *desc);
            Faunus::Energy::Hamiltonian accepted, trial; // State::pot of the two states
            accepted.state = EnergyTerm::MonteCarloState::ACCEPTED;
            trial.state = EnergyTerm::MonteCarloState::TRIAL;
            accepted.maximum_allowed_energy = trial.maximum_allowed_energy = maxenergy;
            accepted.energy_terms.push_back(std::make_shared<faunus_gpu::NonbondedEwaldGPU>(dev));
            trial.energy_terms.push_back(std::make_shared<faunus_gpu::NonbondedEwaldGPU>(dev));
            faunus_gpu::ReferenceStreamMove move(dev, *desc, moves, n_moves, slump_seed, random_seed, false);
            double sum_of_energy_changes = 0.0;
            for (int m = 0; m < n; m++) {
                Change change;
                move.move(change);
                acc_out[m] = 0;
                du_out[m] = 0.0;
                if (!change) continue; // empty move: the reference only draws the Metropolis uniform
                trial.updateState(change);
                const double new_energy = trial.energy(change);
                const double old_energy = accepted.energy(change);
                double du = energy_change(new_energy, old_energy);
                du += move.bias(change, old_energy, new_energy);
                if (std::isnan(du)) throw std::runtime_error("Metropolis error: energy cannot be NaN");
                du_out[m] = du;
                if (metropolis(du, move.uniform())) {
                    accepted.sync(&trial, change);
                    move.accept(change);
                    acc_out[m] = 1;
                }
                else {
                    trial.sync(&accepted, change);
                    move.reject(change);
                    du = 0.0;
                }
                sum_of_energy_changes += du;
            }
            double e = 0.0;
            faunus_gpu::check(fau_get_running_energy(dev->handle(), &e), "fau_get_running_energy");
            energy_out[0] = e;
            energy_out[1] = sum_of_energy_changes;
        }
        fau_ctx_destroy(ctx);
    }
    catch (const std::exception& e) {
        if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", e.what());
        return 1;
    }
    return 0;
}
