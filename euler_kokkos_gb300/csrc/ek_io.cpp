// VTK ImageData output with the reference's own file layout: save_VTK_2D /
// save_VTK_3D of utils/io/IO_VTK.cpp:24-400 (non-MPI builds), reached through
// SolverBase::save_solution -> IO_ReadWrite::save_data (IO_ReadWrite.cpp:50-130).
// The writer reproduces the reference's bytes: the same header text and
// number formatting (C++ stream defaults), the 2D file's version "1.0" and the
// 3D file's "0.1", the raw appended block (a UInt64 byte count before each
// variable, interior cells only, i fastest) or the ASCII form with its
// leading XML declaration, and the file name
// <outputDir>/<outputPrefix>_<step, 7 digits>.vti.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/ek_gb300.h"
#include "ek_internal.h"

namespace
{

// SolverBase::SolverBase (SolverBase.cpp:60-67)
const char * const kVarNames[8] = { "rho", "energy", "rho_vx", "rho_vy", "rho_vz", "bx", "by", "bz" };

bool
big_endian()
{
  const int i = 1;
  return (*(const char *)&i) == 0;
}

} // namespace

extern "C" ek_status
ek_write_vtk(const ek_params * params, const double * U, int layout, int step, const char * debug_name)
{
  using ek_internal::fail;
  if (!params || !U || (layout != EK_LAYOUT_LEFT && layout != EK_LAYOUT_RIGHT) || step < 0)
    return fail(EK_ERR_INVALID, "ek_write_vtk: bad argument");
  const ek_params & p = *params;
  if ((p.dim != 2 && p.dim != 3) || p.nbvar < 1 || p.nbvar > 8)
    return fail(EK_ERR_INVALID, "ek_write_vtk: bad parameters");
  const int  is = p.isize, js = p.jsize, ks = p.dim == 3 ? p.ksize : 1, gw = p.ghost_width;
  const int  nx = p.nx, ny = p.ny, nz = p.dim == 3 ? p.nz : 1, nb = p.nbvar;
  const long plane = (long)is * js, vstride = plane * ks;
  // U(i, j, k, var) in the caller's layout
  auto at = [&](int i, int j, int k, int v) -> double {
    if (layout == EK_LAYOUT_LEFT)
      return U[(long)v * vstride + (long)k * plane + (long)j * is + i];
    return U[(((long)i * js + j) * ks + k) * nb + v];
  };

  std::ostringstream stepNum;
  stepNum.width(7);
  stepNum.fill('0');
  stepNum << step;
  const std::string dir = p.output_dir[0] ? std::string(p.output_dir) : std::string("./");
  const std::string prefix = p.output_prefix[0] ? std::string(p.output_prefix) : std::string("output");
  std::string       filename;
  if (!debug_name || !debug_name[0])
    filename = dir + "/" + prefix + "_" + stepNum.str() + ".vti";
  else
    filename = dir + "/" + prefix + "_" + debug_name + "_" + stepNum.str() + ".vti";

  std::fstream out;
  out.open(filename.c_str(), std::ios_base::out);
  if (!out)
    return fail(EK_ERR_INVALID, "ek_write_vtk: cannot open " + filename);

  const bool ascii = p.vtk_ascii != 0;
  if (ascii)
    out << "<?xml version=\"1.0\"?>\n";
  out << "<VTKFile type=\"ImageData\" version=\"" << (p.dim == 2 ? "1.0" : "0.1") << "\" byte_order=\""
      << (big_endian() ? "BigEndian" : "LittleEndian") << "\" header_type=\"UInt64\">\n";
  if (p.dim == 2)
  {
    out << "  <ImageData WholeExtent=\"" << 0 << " " << nx << " " << 0 << " " << ny << " " << 0 << " " << 0
        << "\" " << "Origin=\"" << p.xmin << " " << p.ymin << " " << 0 << "\" " << "Spacing=\"" << p.dx
        << " " << p.dy << " " << 0.0 << "\">\n";
    out << "  <Piece Extent=\"" << 0 << " " << nx << " " << 0 << " " << ny << " " << 0 << " " << 0 << " "
        << "\">\n";
  }
  else
  {
    out << "  <ImageData WholeExtent=\"" << 0 << " " << nx << " " << 0 << " " << ny << " " << 0 << " " << nz
        << "\" " << "Origin=\"" << p.xmin << " " << p.ymin << " " << p.zmin << "\" " << "Spacing=\"" << p.dx
        << " " << p.dy << " " << p.dz << "\">\n";
    out << "  <Piece Extent=\"" << 0 << " " << nx << " " << 0 << " " << ny << " " << 0 << " " << nz << " "
        << "\">\n";
  }
  out << "    <PointData>\n";
  out << "    </PointData>\n";

  const int k0 = p.dim == 3 ? gw : 0, k1 = p.dim == 3 ? ks - gw : 1;
  if (ascii)
  {
    out << "    <CellData>\n";
    for (int v = 0; v < nb; ++v)
    {
      out << "    <DataArray type=\"Float64\" Name=\"" << kVarNames[v] << "\" format=\"ascii\" >\n";
      for (int k = k0; k < k1; ++k)
        for (int j = gw; j < js - gw; ++j)
          for (int i = gw; i < is - gw; ++i)
            out << at(i, j, k, v) << " ";
      out << "\n    </DataArray>\n";
    }
    out << "    </CellData>\n";
    out << "  </Piece>\n";
    out << "  </ImageData>\n";
    out << "</VTKFile>\n";
  }
  else
  {
    const uint64_t ncells = (uint64_t)nx * ny * nz;
    out << "    <CellData>" << std::endl;
    for (int v = 0; v < nb; ++v)
      out << "     <DataArray type=\"Float64\" Name=\"" << kVarNames[v] << "\" format=\"appended\" offset=\""
          << (uint64_t)v * ncells * sizeof(double) + (uint64_t)v * sizeof(uint64_t) << "\" />" << std::endl;
    out << "    </CellData>" << std::endl;
    out << "  </Piece>" << std::endl;
    out << "  </ImageData>" << std::endl;
    out << "  <AppendedData encoding=\"raw\">" << std::endl;
    out << "_";
    const uint64_t     words = ncells * sizeof(double);
    std::vector<double> row((size_t)nx);
    for (int v = 0; v < nb; ++v)
    {
      out.write((const char *)&words, sizeof(uint64_t));
      for (int k = k0; k < k1; ++k)
        for (int j = gw; j < js - gw; ++j)
        {
          for (int i = 0; i < nx; ++i)
            row[(size_t)i] = at(gw + i, j, k, v);
          out.write((const char *)row.data(), sizeof(double) * (size_t)nx);
        }
    }
    out << "  </AppendedData>" << std::endl;
    out << "</VTKFile>" << std::endl;
  }
  out.close();
  if (!out)
    return fail(EK_ERR_INVALID, "ek_write_vtk: write failed for " + filename);
  return EK_OK;
}
