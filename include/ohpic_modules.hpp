// ohpic_modules.hpp -- C++ mirror of the reference's module API for the particle path,
// over one device-resident context (include/ohpic.h).
//
// The reference's abstract types bind one particle per call:
//   t_ParticleMover%move   src/particle_mover/particle_mover.f90:16-24
//   t_Interpolator%interp  src/interpolator/interpolator.f90:16-25
//   t_Scatter%scatter      src/scatter/scatter.f90:15-24
//   t_FieldSolver%solve    src/field_solver/field_solver.f90:15-25
// and are chosen by string factories (particle_mover_factory.f90:25-30,
// mpi_fft_solver_factory.f90:30-39).  The GPU path keeps the particles on the
// device, so each class here applies its operation to every particle of the
// context ("batched" bindings).  The per-particle forms report
// OHPIC_ERR_UNSUPPORTED.  An unknown factory name is an error, not a silently
// unallocated result as in the reference.
//
// Header-only; errors are thrown as ohpic::Error carrying the status code
// (the reference stops the program with `error stop`).
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "ohpic.h"

namespace ohpic {

class Error : public std::runtime_error {
public:
    Error(int status, const std::string &what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

private:
    int status_;
};

// Owns one ohpic_ctx (device memory and one CUDA stream).
class Context {
public:
    explicit Context(const ohpic_config &cfg)
    {
        const int rc = ohpic_create(&cfg, &ctx_);
        if (rc != OHPIC_OK) throw Error(rc, std::string("ohpic_create: ") + ohpic_status_string(rc));
        nspecies_ = cfg.nspecies;
        n_[0] = cfg.nx;
        n_[1] = cfg.ny;
        n_[2] = cfg.nz;
    }
    ~Context()
    {
        if (ctx_) ohpic_destroy(ctx_);
    }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;

    ohpic_ctx *get() const { return ctx_; }
    int nspecies() const { return nspecies_; }
    long long cells() const { return (long long)n_[0] * n_[1] * n_[2]; }

    void check(int rc, const char *what) const
    {
        if (rc == OHPIC_OK) return;
        char buf[512] = {0};
        ohpic_last_error(ctx_, buf, sizeof(buf));
        throw Error(rc, std::string(what) + ": " + ohpic_status_string(rc) + (buf[0] ? std::string(" (") + buf + ")" : ""));
    }

    // Particle records of one species: oh_particle-like AoS, x,y,z,vx,vy,vz first.
    void upload(int species, const void *pbuf, int64_t n, int64_t stride_bytes)
    {
        check(ohpic_upload_particles(ctx_, species, pbuf, n, stride_bytes), "upload_particles");
    }
    int64_t download(int species, void *pbuf, int64_t capacity, int64_t stride_bytes)
    {
        int64_t n = 0;
        check(ohpic_download_particles(ctx_, species, pbuf, capacity, stride_bytes, &n), "download_particles");
        return n;
    }
    std::vector<double> field(int which)
    {
        std::vector<double> out((size_t)cells());
        check(ohpic_download_field(ctx_, which, out.data()), "download_field");
        return out;
    }
    ohpic_diag diagnostics()
    {
        ohpic_diag d;
        check(ohpic_diagnostics(ctx_, &d), "diagnostics");
        return d;
    }
    void step(double dt, int nsteps) { check(ohpic_step(ctx_, dt, nsteps), "step"); }
    void sort() { check(ohpic_sort(ctx_), "sort"); }

private:
    ohpic_ctx *ctx_ = nullptr;
    int nspecies_ = 0;
    int n_[3] = {0, 0, 0};
};

// t_LinearScatter (linear_scatter.f90:22-55) over every particle.
class Scatter {
public:
    explicit Scatter(Context &c) : c_(c) {}
    void scatter_all() { c_.check(ohpic_scatter(c_.get()), "scatter"); }
    // The per-particle binding is not available on the device path.
    void scatter(const double *particle, double amount, int ps)
    {
        c_.check(ohpic_scatter_one(c_.get(), particle, amount, ps), "scatter_one");
    }

private:
    Context &c_;
};

// t_PoissonFieldSolver (poisson_field_solver.f90:90-175): rho -> phi -> E.
class FieldSolver {
public:
    explicit FieldSolver(Context &c) : c_(c) {}
    void solve() { c_.check(ohpic_solve(c_.get()), "solve"); }

private:
    Context &c_;
};

// t_LinearInterpolator (linear_interpolator.f90:22-69): E at every particle of a species.
class Interpolator {
public:
    explicit Interpolator(Context &c) : c_(c) {}
    std::vector<double> interp_all(int species, int64_t capacity)
    {
        std::vector<double> e((size_t)(3 * capacity));
        int64_t n = 0;
        c_.check(ohpic_interp(c_.get(), species, e.data(), 3 * capacity, &n), "interp");
        e.resize((size_t)(3 * n));
        return e;
    }

private:
    Context &c_;
};

// t_BorisMover (particle_mover_boris.f90:21-64) followed by the periodic wrap,
// applied to every particle without depositing.
class ParticleMover {
public:
    explicit ParticleMover(Context &c) : c_(c) {}
    virtual ~ParticleMover() = default;
    void move_all(double dt) { c_.check(ohpic_move(c_.get(), dt), "move"); }
    void move(double *particle, double qm, const double eb[6], double dt)
    {
        c_.check(ohpic_move_one(c_.get(), particle, qm, eb, dt), "move_one");
    }

private:
    Context &c_;
};

// t_PoissonFieldSolver with a boundary kind per axis (poisson_field_solver.f90:34-175,
// poisson_solver3d.f90:28-207) on the global block 0..n: rho and phi hold
// (n[0]+1)(n[1]+1)(n[2]+1) nodes, x fastest; e three such blocks (or empty).
class BoundedFieldSolver {
public:
    BoundedFieldSolver(const int32_t n[3], const int32_t kinds[3], const double boundary_values[6],
                       int32_t table = OHPIC_TABLE_AS_WRITTEN, int32_t device = 0)
    {
        const int rc = ohpic_poisson_create(n, kinds, boundary_values, table, device, &s_);
        if (rc != OHPIC_OK) throw Error(rc, std::string("ohpic_poisson_create: ") + ohpic_status_string(rc));
    }
    ~BoundedFieldSolver()
    {
        if (s_) ohpic_poisson_destroy(s_);
    }
    BoundedFieldSolver(const BoundedFieldSolver &) = delete;
    BoundedFieldSolver &operator=(const BoundedFieldSolver &) = delete;
    void solve(const double *rho, double *phi, double *e = nullptr)
    {
        const int rc = ohpic_poisson_solve(s_, rho, phi, e);
        if (rc == OHPIC_OK) return;
        char buf[512] = {0};
        ohpic_poisson_last_error(s_, buf, sizeof(buf));
        throw Error(rc, std::string("poisson_solve: ") + ohpic_status_string(rc) + " (" + buf + ")");
    }

private:
    ohpic_poisson *s_ = nullptr;
};

// particle_mover_factory.f90:25-30: "boris" is the only mover.
inline ParticleMover create_particle_mover(const std::string &name, Context &c)
{
    if (name != "boris") throw Error(OHPIC_ERR_INVALID, "unknown particle mover '" + name + "'");
    return ParticleMover(c);
}

}  // namespace ohpic
