// Nektar++ XML/FLD scene loader (hexahedra). Placeholder until the loader
// lands: reports that the format is not supported yet.
#include "ho_host.h"

namespace ho {
int load_xml_fld(const std::string& xml, const std::string& fld, HostScene& hs, std::string& err) {
  (void)xml;
  (void)fld;
  (void)hs;
  err = "XML/FLD loading is not available in this build";
  return HO_ERR_PARSE;
}
}  // namespace ho
