// def.hh of a test flow laid out as DiFfRG's code generator lays out an example's flows/
// directory (flows/def.hh, flows/<dir>/<X>.hh, <X>.cu, <X>.kernel): the same include list at the
// reference's include paths, resolved by the drop-in headers.  Test code of this repository;
// the integrands below are its own.
#pragma once

#include <DiFfRG/common/utils.hh>
#include <DiFfRG/physics/integration.hh>
#include <DiFfRG/physics/integration_finiteT.hh>
#include <DiFfRG/physics/interpolation.hh>
#include <DiFfRG/physics/regulators.hh>
#include <DiFfRG/physics/thermodynamics.hh>

using namespace ::DiFfRG;

struct gen_reg_opts {
  static constexpr int order = 6;
  constexpr static double c = 1.5;
  constexpr static double b0 = 0.25;
};
#define __REGULATOR__ ::DiFfRG::RationalExpRegulator<gen_reg_opts>
