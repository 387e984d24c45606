#ifndef ORACLE_SHIM_CAMP_RESOURCE_HPP
#define ORACLE_SHIM_CAMP_RESOURCE_HPP
namespace camp { namespace resources { struct Host {}; } }
#endif
