// Stand-in for the reference's config/simobject/ElasticMaterialConfig.hpp
// (a yaml-cpp backed class) so that simobject/ElasticMaterial.hpp compiles
// without yaml-cpp. Test infrastructure for oracle/ref/Makefile only: the
// reference's ElasticMaterial is built here through its (name, density, E,
// nu, mu_s, mu_k) constructor, never from a config.
#pragma once
#include <string>

#include "common/types.hpp"

namespace Config {
class ElasticMaterialConfig {
   public:
    std::string name() const { return "config"; }
    Real density() const { return 1000; }
    Real E() const { return 3e3; }
    Real nu() const { return 0.45; }
    Real muS() const { return 0; }
    Real muK() const { return 0; }
};
}  // namespace Config
