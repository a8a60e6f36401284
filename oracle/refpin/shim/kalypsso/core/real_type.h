#pragma once
namespace kalypsso
{
using real_t = double;
}
using kalypsso::real_t;
#define KALYPSSO_NUM(x) static_cast<double>(x)
#define ZERO_F (0.0)
#define ONE_F (1.0)
#define HALF_F (0.5)
#define TWO_F (2.0)
