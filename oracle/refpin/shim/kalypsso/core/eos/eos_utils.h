#pragma once
#include <../better-enums/enum.h>
#include <kalypsso/utils/config/ConfigMap.h>
namespace kalypsso
{
namespace core
{
namespace eos
{
BETTER_ENUM(EOS_TYPE, int, IDEAL_GAS, STIFFENED_GAS)
inline EOS_TYPE
get_eos_type(ConfigMap const &)
{
  return EOS_TYPE::STIFFENED_GAS;
}
} // namespace eos
} // namespace core
} // namespace kalypsso
