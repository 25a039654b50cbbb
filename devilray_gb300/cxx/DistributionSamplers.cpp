// DistributionSamplers.cpp -- generateAliasTable over the device alias build.
#include "tracing/DistributionSamplers.hpp"

AliasTable generateAliasTable(std::span<const float> importances)
{
    AliasTable table{DeviceArray<AliasEntry>((int)importances.size(), AliasEntry{})};
    if (importances.empty()) return table;
    devilray::check(dr_alias_build_host(devilray::context(), importances.data(), (uint32_t)importances.size(),
                                        reinterpret_cast<dr_alias_entry *>(table.entries.hostPtr()), DR_ALIAS_REFERENCE),
                    "generateAliasTable");
    return table;
}
