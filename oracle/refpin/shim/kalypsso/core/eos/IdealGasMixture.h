#pragma once
#include <kalypsso/utils/config/ConfigMap.h>
namespace kalypsso { namespace core { namespace eos {
template <typename device_t>
class IdealGasMixture
{
public:
  IdealGasMixture(ConfigMap const &) {}
};
} } }
