// Files in the reference's formats: restart.bin checkpoints, .vti fields and master.pvd,
// forces.dat / mass_flux.dat and pressure.dat.
//
// Reference (paths inside sakthi-lbm/MRLBM_3D_CUDA):
//   write_checkpoint / read_checkpoint   MRLBM_3D/src/restart/restart_io.cu:3-92
//   write_master_pvd, write_vti_3d, write_vti_3d_annulus
//                                        MRLBM_3D/src/output/saveData.cu:3-231
//   write_forces / write_mass_flux       MRLBM_3D/src/statistics/stat_header.cuh:16-51
//   write_pressure                       MRLBM_3D/src/cases/cylinder/cylinder_kernels.cuh:251-285
//   write_average_inlet_density          MRLBM_3D/src/statistics/stat_header.cuh:53-72
//   write_geometry_files                 MRLBM_3D/src/cases/cylinder/cylinder_helpers.cuh:388-470
// The byte layouts are kept exactly (they are read by the reference's restart path, ParaView
// and post/post.py); values come from this solver's FP64 force sums and FP32 (or decoded
// FP16 / BF16) moments.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include "handle.h"

using namespace mrlbm;

namespace {

int check_device(mrlbm_handle *h) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (!h->initialized) return fail(h, MRLBM_ERR_STATE, "no state yet");
    return MRLBM_OK;
}

// Sampled force rows of `wall` not yet written (all of them when `all`), in step order.
int force_rows(mrlbm_handle *h, int wall, bool all, std::vector<int64_t> &steps, std::vector<double> &f) {
    CK(h, cudaStreamSynchronize(h->stream));
    const int64_t first = std::max<int64_t>(all ? 0 : h->forces_written, h->force_count - kRing);
    const int64_t n = h->force_count - first;
    steps.resize(n);
    f.resize(n * 5);
    std::vector<double> ring((size_t)kRing * 10);
    if (n > 0) CK(h, cudaMemcpy(ring.data(), h->d_force_ring, ring.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int64_t k = 0; k < n; ++k) {
        const int64_t slot = (first + k) % kRing;
        steps[k] = h->force_steps[slot];
        std::memcpy(&f[k * 5], &ring[slot * 10 + wall * 5], 5 * sizeof(double));
    }
    return MRLBM_OK;
}

}  // namespace

extern "C" {

int mrlbm_checkpoint_save(mrlbm_handle *h, const char *path) {
    int rc = check_device(h);
    if (rc) return rc;
    if (!path) return fail(h, MRLBM_ERR_INVALID_ARG, "null path");
    if (h->step > std::numeric_limits<int32_t>::max()) return fail(h, MRLBM_ERR_INVALID_ARG, "step count beyond int32");
    const mrlbm_case_desc &d = h->d;
    std::vector<float> mom((size_t)10 * h->n);
    if ((rc = mrlbm_get_moments(h, MRLBM_FIELD_ALL, MRLBM_LAYOUT_REF_TILED, mom.data(), mom.size())) != MRLBM_OK)
        return rc;
    int64_t len[6], total = 0;
    for (int k = 0; k < 6; ++k) {
        len[k] = halo_face_floats(d.nx, d.ny, d.nz, k / 2);
        total += len[k];
    }
    if ((rc = ensure_stage(h, (size_t)total * sizeof(float))) != MRLBM_OK) return rc;
    float *faces[6];
    for (int k = 0, off = 0; k < 6; off += (int)len[k], ++k) faces[k] = h->d_stage + off;
    CK(h, launch_halo_export(h->d_args, h->parity, h->storage, h->n, faces, h->stream));
    std::vector<float> halo((size_t)total);
    CK(h, cudaMemcpyAsync(halo.data(), h->d_stage, halo.size() * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(h, MRLBM_ERR_IO, std::string("cannot open ") + path);
    const int32_t iter = (int32_t)h->step;
    f.write((const char *)&iter, sizeof(iter));
    f.write((const char *)mom.data(), (std::streamsize)(mom.size() * sizeof(float)));
    f.write((const char *)halo.data(), (std::streamsize)(halo.size() * sizeof(float)));
    if (!f) return fail(h, MRLBM_ERR_IO, std::string("write failed: ") + path);
    return MRLBM_OK;
}

int mrlbm_checkpoint_load(mrlbm_handle *h, const char *path) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (!path) return fail(h, MRLBM_ERR_INVALID_ARG, "null path");
    const mrlbm_case_desc &d = h->d;
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) return fail(h, MRLBM_ERR_IO, std::string("cannot open ") + path);
    const int64_t size = (int64_t)f.tellg();
    int64_t halo = 0;
    for (int k = 0; k < 6; ++k) halo += halo_face_floats(d.nx, d.ny, d.nz, k / 2);
    const int64_t want = 4 + 40 * h->n + 4 * halo;
    if (size != want)
        return fail(h, MRLBM_ERR_IO, std::string(path) + ": " + std::to_string(size) + " bytes, a restart.bin of this grid has " +
                                         std::to_string(want));
    f.seekg(0);
    int32_t iter = 0;
    f.read((char *)&iter, sizeof(iter));
    std::vector<float> mom((size_t)10 * h->n);
    f.read((char *)mom.data(), (std::streamsize)(mom.size() * sizeof(float)));
    if (!f || iter < 0) return fail(h, MRLBM_ERR_IO, std::string("read failed: ") + path);
    // the face populations are the reconstruction of these moments: nothing else to restore
    const int rc = mrlbm_set_moments(h, MRLBM_FIELD_ALL, MRLBM_LAYOUT_REF_TILED, mom.data(), mom.size());
    if (rc) return rc;
    h->step = iter;
    return sync_sr_step(h);
}

int mrlbm_write_vti(mrlbm_handle *h, const char *path) {
    int rc = check_device(h);
    if (rc) return rc;
    if (!path) return fail(h, MRLBM_ERR_INVALID_ARG, "null path");
    const mrlbm_case_desc &d = h->d;
    const int64_t n = h->n;
    std::vector<float> m((size_t)4 * n);
    const uint32_t mask = MRLBM_FIELD_RHO | MRLBM_FIELD_UX | MRLBM_FIELD_UY | MRLBM_FIELD_UZ;
    if ((rc = mrlbm_get_moments(h, mask, MRLBM_LAYOUT_LEXICOGRAPHIC, m.data(), m.size())) != MRLBM_OK) return rc;
    const bool annulus = d.geometry == MRLBM_GEOM_ANNULUS;
    std::vector<std::string> names = annulus ? std::vector<std::string>{"rho", "uz", "u_theta", "u_radial"}
                                             : std::vector<std::string>{"rho", "ux", "uy", "uz"};
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(h, MRLBM_ERR_IO, std::string("cannot open ") + path);
    const uint64_t bytes = (uint64_t)n * sizeof(float);
    f << "<?xml version=\"1.0\"?>\n"
      << "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
      << "  <ImageData WholeExtent=\"0 " << d.nx - 1 << " 0 " << d.ny - 1 << " 0 " << d.nz - 1
      << "\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n"
      << "    <Piece Extent=\"0 " << d.nx - 1 << " 0 " << d.ny - 1 << " 0 " << d.nz - 1 << "\">\n"
      << "      <PointData>\n";
    uint64_t offset = 0;
    for (const std::string &name : names) {
        f << "        <DataArray type=\"Float32\" Name=\"" << name << "\" format=\"appended\" offset=\"" << offset
          << "\"/>\n";
        offset += 8 + bytes;
    }
    f << "      </PointData>\n"
      << "    </Piece>\n"
      << "  </ImageData>\n"
      << "  <AppendedData encoding=\"raw\">\n_";
    const float nan = std::numeric_limits<float>::quiet_NaN();
    const float *rho = m.data(), *ux = rho + n, *uy = ux + n, *uz = uy + n;
    std::vector<float> v((size_t)n);
    auto emit = [&]() {
        f.write((const char *)&bytes, 8);
        f.write((const char *)v.data(), (std::streamsize)bytes);
    };
    auto solid = [&](int64_t i) { return h->geo.cls[i] == C_SOLID; };
    for (int64_t i = 0; i < n; ++i) v[i] = d.rho0 + rho[i];
    emit();
    if (!annulus) {
        for (const float *u : {ux, uy, uz}) {
            for (int64_t i = 0; i < n; ++i) v[i] = solid(i) ? nan : u[i];
            emit();
        }
    } else {
        for (int64_t i = 0; i < n; ++i) v[i] = solid(i) ? nan : uz[i];
        emit();
        // u_theta / u_radial about the axis, normalised by the wall speed scale
        for (int comp = 0; comp < 2; ++comp) {
            for (int64_t i = 0; i < n; ++i) {
                if (solid(i)) {
                    v[i] = nan;
                    continue;
                }
                const int x = (int)(i % d.nx), y = (int)((i / d.nx) % d.ny);
                const float dx = (float)x - d.xc, dy = (float)y - d.yc;
                const float r2 = dx * dx + dy * dy;
                if (r2 < 1e-12f) {
                    v[i] = 0.f;
                    continue;
                }
                const float inv_r = 1.0f / std::sqrt(r2), c = dx * inv_r, s = dy * inv_r;
                v[i] = (comp == 0 ? (-ux[i] * s + uy[i] * c) : (ux[i] * c + uy[i] * s)) / d.u_max;
            }
            emit();
        }
    }
    f << "\n  </AppendedData>\n</VTKFile>\n";
    if (!f) return fail(h, MRLBM_ERR_IO, std::string("write failed: ") + path);
    return MRLBM_OK;
}

int mrlbm_write_master_pvd(const char *path, int32_t macr_save, int32_t max_iter) {
    if (!path || macr_save <= 0 || max_iter < 0) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "bad pvd arguments");
    std::ofstream out(path);
    if (!out) return fail(nullptr, MRLBM_ERR_IO, std::string("cannot open ") + path);
    out << "<VTKFile type=\"Collection\" version=\"0.1\">" << std::endl;
    out << "\t<Collection>" << std::endl;
    for (int it = 0; it <= max_iter; it += macr_save)
        out << "\t\t<DataSet timestep=\"" << it / macr_save << "\" file=\"data" << (10000000 + it) << ".vti\" />"
            << std::endl;
    out << "\t</Collection>" << std::endl;
    out << "</VTKFile>" << std::endl;
    return out ? MRLBM_OK : fail(nullptr, MRLBM_ERR_IO, std::string("write failed: ") + path);
}

int mrlbm_write_forces(mrlbm_handle *h, int32_t wall, const char *forces_path, const char *mass_path, int32_t append) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (wall < 0 || wall > 1 || (!forces_path && !mass_path)) return fail(h, MRLBM_ERR_INVALID_ARG, "bad arguments");
    std::vector<int64_t> steps;
    std::vector<double> f;
    int rc = force_rows(h, wall, append == 0, steps, f);
    if (rc) return rc;
    const auto mode = append ? std::ios::app : std::ios::trunc;
    if (forces_path) {
        std::ofstream out(forces_path, mode);
        if (!out) return fail(h, MRLBM_ERR_IO, std::string("cannot open ") + forces_path);
        out << std::setprecision(16) << std::fixed;
        for (size_t k = 0; k < steps.size(); ++k)
            out << steps[k] << " " << f[k * 5 + 0] << " " << f[k * 5 + 1] << " " << f[k * 5 + 2] << std::endl;
        if (!out) return fail(h, MRLBM_ERR_IO, std::string("write failed: ") + forces_path);
    }
    if (mass_path) {
        std::ofstream out(mass_path, mode);
        if (!out) return fail(h, MRLBM_ERR_IO, std::string("cannot open ") + mass_path);
        out << std::setprecision(16) << std::fixed;
        for (size_t k = 0; k < steps.size(); ++k) out << steps[k] << " " << f[k * 5 + 3] << std::endl;
        if (!out) return fail(h, MRLBM_ERR_IO, std::string("write failed: ") + mass_path);
    }
    h->forces_written = h->force_count;
    return MRLBM_OK;
}

int mrlbm_set_pressure_window(mrlbm_handle *h, int64_t start, int64_t end) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (start >= 0 && end < start) return fail(h, MRLBM_ERR_INVALID_ARG, "window end before start");
    if (start >= 0 && h->geo.n_walls == 0) return fail(h, MRLBM_ERR_UNSUPPORTED, "this case has no curved wall");
    CK(h, cudaStreamSynchronize(h->stream));
    for (int w = 0; w < h->geo.n_walls; ++w) {
        const size_t nb = h->geo.wall[w].list.size();
        if (!h->d_ps_avg[w] && nb > 0) CK(h, cudaMalloc((void **)&h->d_ps_avg[w], nb * sizeof(double)));
        if (nb > 0) CK(h, cudaMemset(h->d_ps_avg[w], 0, nb * sizeof(double)));
    }
    if (!h->d_inlet) CK(h, cudaMalloc((void **)&h->d_inlet, (1 + 2 * kRing) * sizeof(double)));
    CK(h, cudaMemset(h->d_inlet, 0, sizeof(double)));
    h->inlet_steps.assign(kRing, -1);
    h->inlet_written = 0;
    h->ps_start = start < 0 ? -1 : start;
    h->ps_end = start < 0 ? -1 : end;
    h->ps_count = 0;
    return MRLBM_OK;
}

int mrlbm_write_inlet_density(mrlbm_handle *h, const char *path, int32_t append) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (!path || !h->d_inlet) return fail(h, MRLBM_ERR_INVALID_ARG, "no inlet samples (mrlbm_set_pressure_window)");
    CK(h, cudaStreamSynchronize(h->stream));
    const int64_t first = std::max<int64_t>(append ? h->inlet_written : 0, h->ps_count - kRing);
    const int64_t n = h->ps_count - first;
    std::vector<double> e((size_t)std::max<int64_t>(n, 0) * 2);
    for (int64_t c = first; c < h->ps_count; ++c)
        CK(h, cudaMemcpy(&e[(size_t)(c - first) * 2], h->d_inlet + 1 + (c % kRing) * 2, 2 * sizeof(double),
                         cudaMemcpyDeviceToHost));
    std::ofstream out(path, append ? std::ios::app : std::ios::trunc);
    if (!out) return fail(h, MRLBM_ERR_IO, std::string("cannot open ") + path);
    out << std::setprecision(16) << std::fixed;
    for (int64_t k = 0; k < n; ++k)
        out << h->inlet_steps[(size_t)((first + k) % kRing)] << " " << e[(size_t)k * 2] << " " << e[(size_t)k * 2 + 1]
            << std::endl;
    if (!out) return fail(h, MRLBM_ERR_IO, std::string("write failed: ") + path);
    h->inlet_written = h->ps_count;
    return MRLBM_OK;
}

int mrlbm_write_geometry(const mrlbm_handle *h, const char *dir) {
    if (!h || !dir) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null argument");
    static const char *names[9] = {"inner.dat",         "outer.dat",         "bcfluid_inner.dat",
                                   "bcfluid_outer.dat", "bcsolid_inner.dat", "bcsolid_outer.dat",
                                   "solid.dat",         "fluid.dat",         "others.dat"};
    std::ofstream f[9];
    for (int k = 0; k < 9; ++k) {
        const std::string p = std::string(dir) + "/" + names[k];
        f[k].open(p, std::ios::trunc);
        if (!f[k]) return fail(nullptr, MRLBM_ERR_IO, "cannot open " + p);
    }
    const Geometry &g = h->geo;
    const int z = 0;  // the reference writes the z = 0 slice only (Z_SLICE)
    for (int y = 0; y < g.ny; ++y)
        for (int x = 0; x < g.nx; ++x) {
            const int64_t i = x + (int64_t)g.nx * (y + (int64_t)g.ny * z);
            const uint32_t c = g.cls[i], idx = g.payload[i];
            int k;
            switch (c) {
                case C_INNER: k = 0; break;
                case C_OUTER: k = 1; break;
                case C_BCFLUID_INNER: k = 2; break;
                case C_BCFLUID_OUTER: k = 3; break;
                case C_BCSOLID_INNER: k = 4; break;
                case C_BCSOLID_OUTER: k = 5; break;
                default: {
                    // the reference tests (type << index) against NODE_SOLID, then NODE_BULK
                    const uint64_t t = idx < 32 ? (uint64_t)c << idx : ~0ull;
                    k = t == C_SOLID ? 6 : (t == C_BULK ? 7 : 8);
                }
            }
            f[k] << x << " " << y << " " << z << " " << c << " " << idx << "\n";
        }
    for (int k = 0; k < 9; ++k)
        if (!f[k].flush()) return fail(nullptr, MRLBM_ERR_IO, std::string("write failed: ") + names[k]);
    return MRLBM_OK;
}

int mrlbm_write_pressure(mrlbm_handle *h, int32_t wall, const char *path) {
    if (!h) return fail(nullptr, MRLBM_ERR_INVALID_ARG, "null handle");
    if (h->host_only) return fail(h, MRLBM_ERR_STATE, "host-only handle has no device state");
    if (!path || wall < 0 || wall >= h->geo.n_walls || !h->d_ps_avg[wall])
        return fail(h, MRLBM_ERR_INVALID_ARG, "no pressure samples for this wall (mrlbm_set_pressure_window)");
    const WallData &W = h->geo.wall[wall];
    std::vector<double> ps(W.list.size());
    CK(h, cudaStreamSynchronize(h->stream));
    CK(h, cudaMemcpy(ps.data(), h->d_ps_avg[wall], ps.size() * sizeof(double), cudaMemcpyDeviceToHost));
    std::ofstream out(path);
    if (!out) return fail(h, MRLBM_ERR_IO, std::string("cannot open ") + path);
    out << std::setprecision(12);
    out << "theta z Cp\n";
    const mrlbm_case_desc &d = h->d;
    const double kPi = 3.14159265358979323846;
    for (size_t i = 0; i < W.list.size(); ++i) {
        const int64_t node = W.list[i];
        const unsigned x = (unsigned)(node % d.nx), y = (unsigned)((node / d.nx) % d.ny);
        const unsigned z = (unsigned)(node / ((int64_t)d.nx * d.ny));
        const float dx = (float)x - d.xc, dy = (float)y - d.yc;
        float theta = (float)((double)std::atan2(dy, dx) * 180.0 / kPi);
        if (theta < 0) theta = (float)(theta + 360.0);
        out << std::setprecision(12) << theta << " " << z << " " << (float)ps[i] << "\n";
    }
    return out ? MRLBM_OK : fail(h, MRLBM_ERR_IO, std::string("write failed: ") + path);
}

}  // extern "C"
