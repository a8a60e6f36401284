#pragma once
#define KALYPSSO_INFO(...)
#define KALYPSSO_WARN(...)
#define KALYPSSO_ERROR(...)
