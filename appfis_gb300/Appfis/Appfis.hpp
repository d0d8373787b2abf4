/*
 * Appfis.hpp — umbrella header of the GB300 APPFIS engine; applications include it exactly as
 * they include the reference's (Appfis/Appfis.hpp).  The C-ABI library libappfis_gb.so
 * (include/appfis_gb.h) must be linked: -I<repo>/include -L<repo>/appfis_gb300 -lappfis_gb.
 */
#ifndef APPFIS_GB_APPFIS_HPP
#define APPFIS_GB_APPFIS_HPP

#include "Env.hpp"
#include "Attribute.hpp"
#include "Common.hpp"
#include "Utils.hpp"
#include "Array.hpp"
#include "Grid.hpp"
#include "Config.hpp"
#include "Runtime.hpp"
#include "Communication.hpp"
#include "Timer.hpp"

#endif
