// SeisFD3D.conf entries shared by the solver program and the kernel program: the snapshot
// series snap_NNN (io_snap_read / corr_indx / io_snap_locate, code/srcF/mod_io.F90:180-262),
// for one rank holding the whole grid, and the per-rank file-name parts
// (get_fnm_snapnode_n, code/srcF/mod_io.F90:837-846; set_mpi_subfix, code/srcF/mod_mpi.F90:415-423).
#pragma once
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "conf.h"

namespace seisfd {

inline const char* const MPI_SUFFIX = "mpi000000";

inline std::string pad(int v, int width) {
  char b[32];
  std::snprintf(b, sizeof(b), "%0*d", width, v);
  return b;
}

// <root>/<prefix>NNN_mpi000000_nXXXXX.nc
inline std::string snap_file(const std::string& root, const char* prefix, int id, int n) {
  return root + "/" + prefix + pad(id, 3) + "_" + MPI_SUFFIX + "_n" + pad(n, 5) + ".nc";
}

struct SnapDef {
  int id = 0;                      // 1-based snap_NNN number
  int subs[3], subc[3], subt[3];   // subs: 1-based with ghosts
  int gsubs[3], gsube[3];          // interior-relative, as the reference's attributes
  int tinv = 0, tcnt = 0;
  bool vel = false, sgt = false;
};

inline int need_int(const conf::File& cf, const std::string& key, int col) {
  int v;
  if (!cf.get_int(key, col, &v)) throw std::runtime_error("key " + key + " column " + std::to_string(col) + " missing");
  return v;
}

// snap_NNN = subs(3) subc(3) subt(3) tinv tcnt vars, number_of_snap of them; -1 in subs is
// the first interior point, -2 in the k start the free surface, -1 in a count everything
// up to the last interior point.
inline std::vector<SnapDef> read_snaps(const conf::File& cf, int ni, int nj, int nk) {
  std::vector<SnapDef> out;
  const int nsnap = cf.has("number_of_snap") ? need_int(cf, "number_of_snap", 2) : 0;
  const int last[3] = {ni, nj, nk};
  for (int n = 1; n <= nsnap; ++n) {
    const std::string key = "snap_" + pad(n, 3);
    SnapDef sp;
    sp.id = n;
    for (int d = 0; d < 3; ++d) {
      int s0 = need_int(cf, key, d + 2), c0 = need_int(cf, key, d + 5), t0 = need_int(cf, key, d + 8);
      if (s0 == -1) s0 = 1;
      if (d == 2 && s0 == -2) s0 = nk;
      if (t0 < 1) throw std::runtime_error(key + ": stride must be >= 1");
      if (c0 == -1) c0 = (last[d] - s0) / t0 + 1;
      sp.gsubs[d] = s0;
      sp.subc[d] = c0;
      sp.subt[d] = t0;
      sp.gsube[d] = s0 + t0 * (c0 - 1);
      sp.subs[d] = s0 + 3;
    }
    sp.tinv = need_int(cf, key, 11);
    sp.tcnt = need_int(cf, key, 12);
    std::string var;
    if (!cf.get(key, 13, &var)) throw std::runtime_error(key + ": variable list (V, T or TV) missing");
    sp.vel = var.find('V') != std::string::npos;
    sp.sgt = var.find('T') != std::string::npos;
    if (sp.tinv < 1 || sp.tcnt < 1) throw std::runtime_error(key + ": tinv and tcnt must be >= 1");
    out.push_back(sp);
  }
  return out;
}

}  // namespace seisfd
