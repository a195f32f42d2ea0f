// pybind11 module that exposes the reference's OWN evaluator and flow-field
// functors, compiled in place from the azplugins source tree (include path only,
// nothing copied). It is the pin for the oracle restatement in azp_oracle.cpp:
// tests compare the two on random inputs, and tests/golden/make_ref_vectors.py
// records its outputs as fixtures that travel without the reference.
//
// Test infrastructure only: built into oracle/_ref/ by oracle/build_ref.sh, never
// imported by the product.
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include "BondEvaluatorDoubleWell.h"
#include "BondEvaluatorQuartic.h"
#include "ConstantFlow.h"
#include "PairEvaluatorColloid.h"
#include "PairEvaluatorExpandedYukawa.h"
#include "PairEvaluatorHertz.h"
#include "PairEvaluatorPerturbedLennardJones.h"
#include "ParabolicFlow.h"

// the flow-field headers undefine pybind11's export macro on their way out
#ifndef PYBIND11_EXPORT
#define PYBIND11_EXPORT __attribute__((visibility("default")))
#endif

#include <string>
#include <tuple>
#include <vector>

namespace py = pybind11;
namespace az = hoomd::azplugins;
namespace azd = hoomd::azplugins::detail;

template<class Eval> static py::tuple pair_eval(py::dict d, double rsq, double rcutsq, bool shift)
    {
    typename Eval::param_type p(d);
    Eval ev(rsq, rcutsq, p);
    double f = 0.0, e = 0.0;
    bool ok = ev.evalForceAndEnergy(f, e, shift);
    return py::make_tuple(ok, f, e);
    }

template<class Eval> static py::tuple bond_eval(py::dict d, double rsq)
    {
    typename Eval::param_type p(d);
    Eval ev(rsq, p);
    double f = 0.0, e = 0.0;
    bool ok = ev.evalForceAndEnergy(f, e);
    return py::make_tuple(ok, f, e);
    }

template<class P> static py::dict roundtrip(py::dict d)
    {
    P p(d);
    return p.asDict();
    }

// raw param_type fields, in declaration order
static std::vector<double> raw_pair(const std::string& name, py::dict d)
    {
    if (name == "PerturbedLennardJones")
        {
        azd::PairParametersPerturbedLennardJones p(d);
        return {p.sigma_6, p.epsilon_x_4, p.attraction_scale_factor, p.rwcasq};
        }
    if (name == "ExpandedYukawa")
        {
        azd::PairParametersExpandedYukawa p(d);
        return {p.epsilon, p.kappa, p.delta};
        }
    if (name == "Hertz")
        {
        azd::PairParametersHertz p(d);
        return {p.epsilon};
        }
    if (name == "Colloid")
        {
        azd::PairParametersColloid p(d);
        return {p.A, p.a_1, p.a_2, p.sigma_3};
        }
    throw std::runtime_error("unknown pair evaluator " + name);
    }

static std::vector<double> raw_bond(const std::string& name, py::dict d)
    {
    if (name == "Quartic")
        {
        azd::BondParametersQuartic p(d);
        return {p.k, p.r_0, p.b_1, p.b_2, p.U_0, p.sigma_6, p.epsilon_x_4, p.delta};
        }
    if (name == "DoubleWell")
        {
        azd::BondParametersDoubleWell p(d);
        return {p.r_1, p.r_diff, p.U_1, p.U_tilt};
        }
    throw std::runtime_error("unknown bond evaluator " + name);
    }

PYBIND11_MODULE(azp_ref, m)
    {
    m.doc() = "reference azplugins evaluators compiled in place (oracle pin)";
    m.def("pair_eval",
          [](const std::string& name, py::dict d, double rsq, double rcutsq, bool shift)
          {
              if (name == "PerturbedLennardJones")
                  return pair_eval<azd::PairEvaluatorPerturbedLennardJones>(d, rsq, rcutsq, shift);
              if (name == "ExpandedYukawa")
                  return pair_eval<azd::PairEvaluatorExpandedYukawa>(d, rsq, rcutsq, shift);
              if (name == "Hertz")
                  return pair_eval<azd::PairEvaluatorHertz>(d, rsq, rcutsq, shift);
              if (name == "Colloid")
                  return pair_eval<azd::PairEvaluatorColloid>(d, rsq, rcutsq, shift);
              throw std::runtime_error("unknown pair evaluator " + name);
          });
    m.def("bond_eval",
          [](const std::string& name, py::dict d, double rsq)
          {
              if (name == "Quartic")
                  return bond_eval<azd::BondEvaluatorQuartic>(d, rsq);
              if (name == "DoubleWell")
                  return bond_eval<azd::BondEvaluatorDoubleWell>(d, rsq);
              throw std::runtime_error("unknown bond evaluator " + name);
          });
    m.def("pair_roundtrip",
          [](const std::string& name, py::dict d)
          {
              if (name == "PerturbedLennardJones")
                  return roundtrip<azd::PairParametersPerturbedLennardJones>(d);
              if (name == "ExpandedYukawa")
                  return roundtrip<azd::PairParametersExpandedYukawa>(d);
              if (name == "Hertz")
                  return roundtrip<azd::PairParametersHertz>(d);
              if (name == "Colloid")
                  return roundtrip<azd::PairParametersColloid>(d);
              throw std::runtime_error("unknown pair evaluator " + name);
          });
    m.def("bond_roundtrip",
          [](const std::string& name, py::dict d)
          {
              if (name == "Quartic")
                  return roundtrip<azd::BondParametersQuartic>(d);
              if (name == "DoubleWell")
                  return roundtrip<azd::BondParametersDoubleWell>(d);
              throw std::runtime_error("unknown bond evaluator " + name);
          });
    m.def("pair_raw", &raw_pair);
    m.def("bond_raw", &raw_bond);
    m.def("constant_flow",
          [](std::tuple<double, double, double> U, std::tuple<double, double, double> r)
          {
              az::ConstantFlow f(hoomd::make_scalar3(std::get<0>(U), std::get<1>(U), std::get<2>(U)));
              hoomd::Scalar3 u = f(hoomd::make_scalar3(std::get<0>(r), std::get<1>(r), std::get<2>(r)));
              return std::make_tuple(u.x, u.y, u.z);
          });
    m.def("parabolic_flow",
          [](double mean_velocity, double separation, std::tuple<double, double, double> r)
          {
              az::ParabolicFlow f(mean_velocity, separation);
              hoomd::Scalar3 u = f(hoomd::make_scalar3(std::get<0>(r), std::get<1>(r), std::get<2>(r)));
              return std::make_tuple(u.x, u.y, u.z, f.getMeanVelocity(), f.getSeparation());
          });
    }
