// Included by the reference's src/lbm.hpp; nothing from it is used.
#pragma once
#include "Kokkos_Core.hpp"
