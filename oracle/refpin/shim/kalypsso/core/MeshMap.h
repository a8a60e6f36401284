// forwards to the core stand-ins of shim_core.h
#pragma once
#include <kalypsso/core/shim_core.h>
