// C++ drop-in for the reference header library's step API (SolverBase,
// ParkerSolver, FocusTransportSolver / FocusSolver, ParticleSystem, Field,
// RandomManager, the coefficient builders), header-only over libkpt's C ABI.
// Link with -lkpt.
#pragma once

#include "Coefficients.hpp"
#include "FocusSolver.hpp"
#include "Grid.hpp"
#include "ParkerSolver.hpp"
#include "ParticleSystem.hpp"
#include "RandomManager.hpp"
#include "Runtime.hpp"
#include "SolverBase.hpp"
