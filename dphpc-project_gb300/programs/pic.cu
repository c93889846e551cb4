// Particle-in-cell mini-app as an MPI program (converter-output form),
// written for this runtime (the reference runs sputniPIC; nothing of it is
// used here beyond the idea of a thermal plasma with u_th = 0.045).
//
// 2D electromagnetic PIC on a periodic GX x GY grid (cell size 1, c = 1):
// fields Ex, Ey, Bz on a Yee mesh, explicit leapfrog (dt = 0.5); particles of
// two species (electrons q/m = -1, ions q/m = +1/25) with positions and two
// velocity components, pushed with the Boris rotation; currents deposited by
// cloud-in-cell weights.  Ranks own PX x PY blocks of the grid:
//   * field ghost cells travel with MPI_Sendrecv (x first, then y, so corners
//     come along), and ghost currents are sent back and added the same way;
//   * particles that leave the block go to one of the 8 neighbours with
//     MPI_Isend / MPI_Irecv of counts and then of malloc'd variable-size
//     buffers;
//   * kinetic and field energies are summed with MPI_Allreduce.
//
// The particle and grid loops run through gpumpi_parallel_for (omp.h.cuh):
// on the GPU over the rank's whole thread block, in a host build in order.
// Both give the same bits because nothing depends on the order in which
// iterations run: particles are dealt into `nchunk` fixed chunks (chunk c holds
// particles c, c + nchunk, c + 2 nchunk, ...: neighbouring threads read
// neighbouring particles) whatever the thread count, energies are summed per
// chunk and the chunks' sums added in chunk order, stayers and leavers are
// written chunk by chunk at offsets from the chunks' counts, and currents are
// deposited in 64-bit fixed point (2^-40 units, truncated), whose sums are
// exact in any order (gpumpi_atomic_add_i64: an atomic add on the GPU, a plain
// add on the host).
//
// Initial state: PPC particles per cell and species at seeded uniform
// positions, thermal velocities by the Irwin-Hall sum of 12 uniforms (only
// additions), electrons in two counter-streaming beams (+-0.1) so that
// particles migrate.  All arithmetic is + - * / on doubles in a fixed order:
// a GPU run (-fmad=false) and a host MPI run give the same bits.
// Rank 0 prints the energies every `report` cycles and a checksum of all
// particle positions at the end.
// Usage: pic [cycles=50] [GX=256] [GY=128] [PPC=125] [report=10] [nchunk=1024]
//        (P ranks as PX x PY with PX >= PY, the most square split)
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"
#include "omp.h.cuh"

#define NSPEC 2

__device__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ double unif(unsigned long long* s) {
    *s += 0x9E3779B97F4A7C15ull;
    return (double)(mix64(*s) >> 11) * (1.0 / 9007199254740992.0);
}

// Particles of one species on one rank (structure of arrays).
struct Species {
    double* x;
    double* y;
    double* u;
    double* v;
    long n;
    long cap;
    double* ax;     // spare arrays: the compaction target, swapped with x..v
    double* ay;
    double* au;
    double* av;
    long alt_cap;
    double qm;      // charge / mass
    double qw;      // charge of one macro-particle
    double mw;      // mass of one macro-particle
};

// Everything the parallel loops read or write, in the heap.
struct Pic {
    // grid: (nx+2) x (ny+2) with one ghost layer, index (i+1) + (j+1)*(nx+2)
    int nx, ny, x0, y0, GX, GY, PX, PY, bx, by, cells, nchunk;
    double dt;
    double* ex;
    double* ey;
    double* bz;
    double* jx;
    double* jy;
    long long* ajx;          // [cells] fixed-point current accumulators
    long long* ajy;
    double* part;            // [nchunk][4] per-chunk partial sums
    Species sp[NSPEC];
    int s;                   // species of the running loop
    // migration
    signed char* dest;       // [n] neighbour index 0..7 of each particle, -1 = stays
    int* ccount;             // [nchunk][9] per chunk: leavers per neighbour, stayers
    long* coff;              // [nchunk][9] write offsets
    double* sbuf[8];         // outgoing particles per neighbour (4 doubles each)
    double* rbq[8];          // incoming particles per neighbour
    long roff[9];            // their offsets in the appended run (prefix of the counts)
    long app_base;           // first index of the appended run
    long qtot[9];            // leavers per neighbour, stayers (sums over the chunks)
};

__device__ int gid(const Pic* g, int i, int j) { return (i + 1) + (j + 1) * (g->nx + 2); }

__device__ int reserve(Species* s, long need) {
    if (need <= s->cap) return 0;
    long cap = need + need / 2 + 64;
    double* nx = (double*)malloc(sizeof(double) * cap);
    double* ny = (double*)malloc(sizeof(double) * cap);
    double* nu = (double*)malloc(sizeof(double) * cap);
    double* nv = (double*)malloc(sizeof(double) * cap);
    if (!nx || !ny || !nu || !nv) return 1;
    if (s->n) {
        memcpy(nx, s->x, sizeof(double) * s->n);
        memcpy(ny, s->y, sizeof(double) * s->n);
        memcpy(nu, s->u, sizeof(double) * s->n);
        memcpy(nv, s->v, sizeof(double) * s->n);
    }
    free(s->x);
    free(s->y);
    free(s->u);
    free(s->v);
    s->x = nx;
    s->y = ny;
    s->u = nu;
    s->v = nv;
    s->cap = cap;
    return 0;
}

// Rank of the block at (bx, by) with periodic wrap.
__device__ int block_rank(int bx, int by, int PX, int PY) {
    bx = (bx + PX) % PX;
    by = (by + PY) % PY;
    return bx + by * PX;
}

// Copy ghost layers of field f: x direction (columns), then y (rows incl. ghost columns).
__device__ void halo_fill(Pic* g, double* f, double* sb, double* rb, int left, int right, int down, int up) {
    const int nx = g->nx, ny = g->ny, W = nx + 2;
    for (int j = 0; j < ny; j++) sb[j] = f[gid(g, nx - 1, j)];
    MPI_Sendrecv(sb, ny, MPI_DOUBLE, right, 11, rb, ny, MPI_DOUBLE, left, 11, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int j = 0; j < ny; j++) f[gid(g, -1, j)] = rb[j];
    for (int j = 0; j < ny; j++) sb[j] = f[gid(g, 0, j)];
    MPI_Sendrecv(sb, ny, MPI_DOUBLE, left, 12, rb, ny, MPI_DOUBLE, right, 12, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int j = 0; j < ny; j++) f[gid(g, nx, j)] = rb[j];
    for (int i = -1; i <= nx; i++) sb[i + 1] = f[gid(g, i, ny - 1)];
    MPI_Sendrecv(sb, W, MPI_DOUBLE, up, 13, rb, W, MPI_DOUBLE, down, 13, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int i = -1; i <= nx; i++) f[gid(g, i, -1)] = rb[i + 1];
    for (int i = -1; i <= nx; i++) sb[i + 1] = f[gid(g, i, 0)];
    MPI_Sendrecv(sb, W, MPI_DOUBLE, down, 14, rb, W, MPI_DOUBLE, up, 14, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int i = -1; i <= nx; i++) f[gid(g, i, ny)] = rb[i + 1];
}

// Add ghost contributions of f to the owners: y rows first (incl. ghost columns), then x columns.
__device__ void halo_add(Pic* g, double* f, double* sb, double* rb, int left, int right, int down, int up) {
    const int nx = g->nx, ny = g->ny, W = nx + 2;
    for (int i = -1; i <= nx; i++) sb[i + 1] = f[gid(g, i, ny)];
    MPI_Sendrecv(sb, W, MPI_DOUBLE, up, 21, rb, W, MPI_DOUBLE, down, 21, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int i = -1; i <= nx; i++) f[gid(g, i, 0)] = f[gid(g, i, 0)] + rb[i + 1];
    for (int i = -1; i <= nx; i++) sb[i + 1] = f[gid(g, i, -1)];
    MPI_Sendrecv(sb, W, MPI_DOUBLE, down, 22, rb, W, MPI_DOUBLE, up, 22, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int i = -1; i <= nx; i++) f[gid(g, i, ny - 1)] = f[gid(g, i, ny - 1)] + rb[i + 1];
    for (int j = 0; j < ny; j++) sb[j] = f[gid(g, nx, j)];
    MPI_Sendrecv(sb, ny, MPI_DOUBLE, right, 23, rb, ny, MPI_DOUBLE, left, 23, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int j = 0; j < ny; j++) f[gid(g, 0, j)] = f[gid(g, 0, j)] + rb[j];
    for (int j = 0; j < ny; j++) sb[j] = f[gid(g, -1, j)];
    MPI_Sendrecv(sb, ny, MPI_DOUBLE, left, 24, rb, ny, MPI_DOUBLE, right, 24, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int j = 0; j < ny; j++) f[gid(g, nx - 1, j)] = f[gid(g, nx - 1, j)] + rb[j];
}

// Cloud-in-cell weights of a position relative to the local block.
__device__ void cic(const Pic* g, double px, double py, int* i, int* j, double* fx, double* fy) {
    const double lx = px - (double)g->x0, ly = py - (double)g->y0;
    int ii = (int)lx, jj = (int)ly;
    if (lx < 0.0) ii = -1;
    if (ly < 0.0) jj = -1;
    if (ii > g->nx - 1) ii = g->nx - 1;
    if (jj > g->ny - 1) jj = g->ny - 1;
    *i = ii;
    *j = jj;
    *fx = lx - (double)ii;
    *fy = ly - (double)jj;
}

__device__ double interp(const Pic* g, const double* f, int i, int j, double fx, double fy) {
    const double a = f[gid(g, i, j)] * (1.0 - fx) + f[gid(g, i + 1, j)] * fx;
    const double b = f[gid(g, i, j + 1)] * (1.0 - fx) + f[gid(g, i + 1, j + 1)] * fx;
    return a * (1.0 - fy) + b * fy;
}

// ---- loop bodies (one call per chunk, cell or row) ----

__device__ void push_chunk(long c, void* arg) {
    Pic* g = (Pic*)arg;
    Species* S = &g->sp[g->s];
    const double dt = g->dt;
    const double h = 0.5 * S->qm * dt;
    double* x = S->x;
    double* y = S->y;
    double* u = S->u;
    double* v = S->v;
    const long n = S->n, step = g->nchunk;
    const double GXd = (double)g->GX, GYd = (double)g->GY;
    for (long k = c; k < n; k += step) {
        int i, j;
        double fx, fy;
        const double px = x[k], py = y[k];
        cic(g, px, py, &i, &j, &fx, &fy);
        const double ex = interp(g, g->ex, i, j, fx, fy);
        const double ey = interp(g, g->ey, i, j, fx, fy);
        const double bz = interp(g, g->bz, i, j, fx, fy);
        // Boris: half kick, rotation about z, half kick
        double um = u[k] + h * ex, vm = v[k] + h * ey;
        const double t = h * bz;
        const double sfac = 2.0 * t / (1.0 + t * t);
        const double up_ = um + vm * t, vp_ = vm - um * t;
        um = um + vp_ * sfac;
        vm = vm - up_ * sfac;
        const double un = um + h * ex, vn = vm + h * ey;
        u[k] = un;
        v[k] = vn;
        double nxp = px + un * dt, nyp = py + vn * dt;
        if (nxp < 0.0) nxp += GXd;
        if (nxp >= GXd) nxp -= GXd;
        if (nyp < 0.0) nyp += GYd;
        if (nyp >= GYd) nyp -= GYd;
        x[k] = nxp;
        y[k] = nyp;
    }
}

// Neighbour index (0..7) of every particle that left the block, -1 for the rest.
__device__ void classify_chunk(long c, void* arg) {
    Pic* g = (Pic*)arg;
    Species* S = &g->sp[g->s];
    int* cnt = g->ccount + c * 9;
    int loc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double* x = S->x;
    const double* y = S->y;
    signed char* dest = g->dest;
    const long n = S->n, step = g->nchunk;
    for (long k = c; k < n; k += step) {
        const int cx = (int)x[k] / g->nx, cy = (int)y[k] / g->ny;
        int dx = cx - g->bx, dy = cy - g->by;
        if (dx > 1) dx -= g->PX;
        if (dx < -1) dx += g->PX;
        if (dy > 1) dy -= g->PY;
        if (dy < -1) dy += g->PY;
        int q = -1;
        if (dx != 0 || dy != 0) {
            q = (dy + 1) * 3 + (dx + 1);
            if (q > 4) q--;
        }
        dest[k] = (signed char)q;
        loc[q < 0 ? 8 : q]++;
    }
    for (int q = 0; q < 9; q++) cnt[q] = loc[q];
}

// Leavers go to their neighbour's buffer, stayers to the compacted arrays,
// each at the offsets of its chunk (chunk-major order, the same in every build).
__device__ void scatter_chunk(long c, void* arg) {
    Pic* g = (Pic*)arg;
    Species* S = &g->sp[g->s];
    long off[9];
    for (int q = 0; q < 9; q++) off[q] = g->coff[c * 9 + q];
    const double* x = S->x;
    const double* y = S->y;
    const double* u = S->u;
    const double* v = S->v;
    double* ax = S->ax;
    double* ay = S->ay;
    double* au = S->au;
    double* av = S->av;
    const signed char* dest = g->dest;
    const long n = S->n, step = g->nchunk;
    for (long k = c; k < n; k += step) {
        const int q = dest[k];
        if (q < 0) {
            const long w = off[8]++;
            ax[w] = x[k];
            ay[w] = y[k];
            au[w] = u[k];
            av[w] = v[k];
        } else {
            double* d = g->sbuf[q] + 4 * off[q]++;
            d[0] = x[k];
            d[1] = y[k];
            d[2] = u[k];
            d[3] = v[k];
        }
    }
}

#define FIX_ONE 1099511627776.0   // 2^40

__device__ void deposit_fixed(const Pic* g, long long* f, int i, int j, double fx, double fy, double val) {
    gpumpi_atomic_add_i64(&f[gid(g, i, j)], (long long)(val * (1.0 - fx) * (1.0 - fy) * FIX_ONE));
    gpumpi_atomic_add_i64(&f[gid(g, i + 1, j)], (long long)(val * fx * (1.0 - fy) * FIX_ONE));
    gpumpi_atomic_add_i64(&f[gid(g, i, j + 1)], (long long)(val * (1.0 - fx) * fy * FIX_ONE));
    gpumpi_atomic_add_i64(&f[gid(g, i + 1, j + 1)], (long long)(val * fx * fy * FIX_ONE));
}

// Destination q (0..7 a neighbour, 8 the stayers): every chunk's write offset
// is the sum of the earlier chunks' counts.  Eight counts are read before any
// offset is written, so the reads do not wait on the writes.
__device__ void chunk_offsets_q(long q, void* arg) {
    Pic* g = (Pic*)arg;
    const int nch = g->nchunk;
    const int* cnt = g->ccount;
    long* off = g->coff;
    long run = 0;
    for (int c = 0; c < nch; c += 8) {
        const int m = nch - c < 8 ? nch - c : 8;
        int v[8];
        for (int k = 0; k < m; k++) v[k] = cnt[(c + k) * 9 + (int)q];
        for (int k = 0; k < m; k++) {
            off[(c + k) * 9 + (int)q] = run;
            run += v[k];
        }
    }
    g->qtot[q] = run;
}

// Incoming particle i (neighbour-major order) appended after the stayers.
__device__ void append_particle(long i, void* arg) {
    Pic* g = (Pic*)arg;
    Species* S = &g->sp[g->s];
    int q = 0;
    while (i >= g->roff[q + 1]) q++;
    const double* d = g->rbq[q] + 4 * (i - g->roff[q]);
    const long k = g->app_base + i;
    S->x[k] = d[0];
    S->y[k] = d[1];
    S->u[k] = d[2];
    S->v[k] = d[3];
}

__device__ void clear_current_cell(long k, void* arg) {
    Pic* g = (Pic*)arg;
    g->ajx[k] = 0;
    g->ajy[k] = 0;
}

// Deposit of one chunk of both species into the fixed-point accumulators.
__device__ void deposit_chunk(long c, void* arg) {
    Pic* g = (Pic*)arg;
    for (int s = 0; s < NSPEC; s++) {
        const Species* S = &g->sp[s];
        const double* x = S->x;
        const double* y = S->y;
        const double* u = S->u;
        const double* v = S->v;
        const double qw = S->qw;
        const long n = S->n, step = g->nchunk;
        for (long k = c; k < n; k += step) {
            int i, j;
            double fx, fy;
            cic(g, x[k], y[k], &i, &j, &fx, &fy);
            deposit_fixed(g, g->ajx, i, j, fx, fy, qw * u[k]);
            deposit_fixed(g, g->ajy, i, j, fx, fy, qw * v[k]);
        }
    }
}

__device__ void current_from_fixed_cell(long k, void* arg) {
    Pic* g = (Pic*)arg;
    g->jx[k] = (double)g->ajx[k] * (1.0 / FIX_ONE);
    g->jy[k] = (double)g->ajy[k] * (1.0 / FIX_ONE);
}

__device__ void bz_half_row(long j, void* arg) {
    Pic* g = (Pic*)arg;
    for (int i = 0; i < g->nx; i++) {
        const double curl = (g->ey[gid(g, i + 1, (int)j)] - g->ey[gid(g, i, (int)j)]) -
                            (g->ex[gid(g, i, (int)j + 1)] - g->ex[gid(g, i, (int)j)]);
        g->bz[gid(g, i, (int)j)] -= 0.5 * g->dt * curl;
    }
}

__device__ void e_full_row(long j, void* arg) {
    Pic* g = (Pic*)arg;
    for (int i = 0; i < g->nx; i++) {
        const int c = gid(g, i, (int)j);
        g->ex[c] += g->dt * ((g->bz[c] - g->bz[gid(g, i, (int)j - 1)]) - g->jx[c]);
        g->ey[c] += g->dt * (-(g->bz[c] - g->bz[gid(g, i - 1, (int)j)]) - g->jy[c]);
    }
}

// Per-chunk kinetic sums (both species) and per-row field sums.
__device__ void energy_chunk(long c, void* arg) {
    Pic* g = (Pic*)arg;
    double* e = g->part + c * 4;
    for (int s = 0; s < NSPEC; s++) {
        const Species* S = &g->sp[s];
        const double* u = S->u;
        const double* v = S->v;
        const long n = S->n, step = g->nchunk;
        double ke = 0.0;
        for (long k = c; k < n; k += step) ke += u[k] * u[k] + v[k] * v[k];
        e[s] = ke;
    }
    e[2] = 0.0;
    e[3] = 0.0;
    if (c < g->ny) {
        for (int i = 0; i < g->nx; i++) {
            const int q = gid(g, i, (int)c);
            e[2] += g->ex[q] * g->ex[q] + g->ey[q] * g->ey[q];
            e[3] += g->bz[q] * g->bz[q];
        }
    }
}

__device__ int __gpu_main(int argc, char** argv) {
    int rank, size;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    const int cycles = argc > 1 ? atoi(argv[1]) : 50;
    const int GX = argc > 2 ? atoi(argv[2]) : 256;
    const int GY = argc > 3 ? atoi(argv[3]) : 128;
    const int PPC = argc > 4 ? atoi(argv[4]) : 125;
    const int report = argc > 5 ? atoi(argv[5]) : 10;
    int nchunk = argc > 6 ? atoi(argv[6]) : 1024;
    // process grid: the most square PX x PY with PX >= PY
    int PY = 1;
    for (int d = 1; d * d <= size; d++)
        if (size % d == 0) PY = d;
    const int PX = size / PY;
    if (GX % PX || GY % PY) {
        if (rank == 0) printf("pic: grid %dx%d does not split over %dx%d ranks\n", GX, GY, PX, PY);
        MPI_Finalize();
        return 1;
    }
    Pic* g = (Pic*)calloc(1, sizeof(Pic));
    g->PX = PX;
    g->PY = PY;
    g->bx = rank % PX;
    g->by = rank / PX;
    g->nx = GX / PX;
    g->ny = GY / PY;
    g->x0 = g->bx * g->nx;
    g->y0 = g->by * g->ny;
    g->GX = GX;
    g->GY = GY;
    g->dt = 0.5;
    if (nchunk < g->ny) nchunk = g->ny;   // energy rows ride on the chunk loop
    g->nchunk = nchunk;
    g->cells = (g->nx + 2) * (g->ny + 2);
    double* fields = (double*)calloc((size_t)g->cells * 5, sizeof(double));
    g->ex = fields;
    g->ey = fields + g->cells;
    g->bz = fields + 2 * g->cells;
    g->jx = fields + 3 * g->cells;
    g->jy = fields + 4 * g->cells;
    g->ajx = (long long*)malloc(sizeof(long long) * 2 * (size_t)g->cells);
    g->ajy = g->ajx + g->cells;
    g->part = (double*)malloc(sizeof(double) * 4 * nchunk);
    g->ccount = (int*)malloc(sizeof(int) * 9 * nchunk);
    g->coff = (long*)malloc(sizeof(long) * 9 * nchunk);
    const int hb = (g->nx > g->ny ? g->nx : g->ny) + 2;
    double* sb = (double*)malloc(sizeof(double) * hb);
    double* rb = (double*)malloc(sizeof(double) * hb);
    const int bx = g->bx, by = g->by;
    const int left = block_rank(bx - 1, by, PX, PY), right = block_rank(bx + 1, by, PX, PY);
    const int down = block_rank(bx, by - 1, PX, PY), up = block_rank(bx, by + 1, PX, PY);
    int nb[8];
    {
        int k = 0;
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++)
                if (dx || dy) nb[k++] = block_rank(bx + dx, by + dy, PX, PY);
    }
    const double uth[NSPEC] = {0.045, 0.009};
    const double qm[NSPEC] = {-1.0, 1.0 / 25.0};
    // plasma frequency 0.1 for electrons: density 1 per cell, w_p^2 = q^2 n / m
    const double qe = 0.1 / (double)PPC;
    int status = 0;
    long dest_cap = 0;
    for (int s = 0; s < NSPEC; s++) {
        Species* S = &g->sp[s];
        S->qm = qm[s];
        S->qw = s == 0 ? -qe : qe;
        S->mw = S->qw / S->qm;
        if (reserve(S, (long)g->nx * g->ny * PPC + 64)) status = 1;
        unsigned long long seed = mix64(((unsigned long long)rank << 8) + (unsigned long long)s + 1);
        for (int j = 0; j < g->ny && !status; j++)
            for (int i = 0; i < g->nx; i++)
                for (int p = 0; p < PPC; p++) {
                    const long k = S->n++;
                    S->x[k] = (double)(g->x0 + i) + unif(&seed);
                    S->y[k] = (double)(g->y0 + j) + unif(&seed);
                    double a = 0.0, b = 0.0;
                    for (int q = 0; q < 12; q++) a += unif(&seed);
                    for (int q = 0; q < 12; q++) b += unif(&seed);
                    S->u[k] = (a - 6.0) * uth[s] + (s == 0 ? ((p & 1) ? 0.1 : -0.1) : 0.0);
                    S->v[k] = (b - 6.0) * uth[s];
                }
    }
    MPI_Barrier(MPI_COMM_WORLD);
    const double t0 = MPI_Wtime();
    for (int cyc = 1; cyc <= cycles && !status; cyc++) {
        // 1. push and move
        halo_fill(g, g->ex, sb, rb, left, right, down, up);
        halo_fill(g, g->ey, sb, rb, left, right, down, up);
        halo_fill(g, g->bz, sb, rb, left, right, down, up);
        for (int s = 0; s < NSPEC; s++) {
            g->s = s;
            gpumpi_parallel_for(nchunk, push_chunk, g);
        }
        // 2. migrate particles that left the block, species by species
        for (int s = 0; s < NSPEC && !status; s++) {
            Species* S = &g->sp[s];
            g->s = s;
            if (S->n > dest_cap) {
                free(g->dest);
                dest_cap = S->cap;
                g->dest = (signed char*)malloc(dest_cap);
                if (!g->dest) {
                    status = 1;
                    break;
                }
            }
            if (S->n > S->alt_cap) {   // the stayers (at most n) are written to the spare arrays
                free(S->ax);
                free(S->ay);
                free(S->au);
                free(S->av);
                S->alt_cap = S->cap;
                S->ax = (double*)malloc(sizeof(double) * S->alt_cap);
                S->ay = (double*)malloc(sizeof(double) * S->alt_cap);
                S->au = (double*)malloc(sizeof(double) * S->alt_cap);
                S->av = (double*)malloc(sizeof(double) * S->alt_cap);
                if (!S->ax || !S->ay || !S->au || !S->av) {
                    status = 1;
                    break;
                }
            }
            gpumpi_parallel_for(nchunk, classify_chunk, g);
            int scnt[8], rcnt[8];
            gpumpi_parallel_for(9, chunk_offsets_q, g);
            for (int q = 0; q < 8; q++) scnt[q] = (int)g->qtot[q];
            const long stay = g->qtot[8];
            for (int q = 0; q < 8; q++) g->sbuf[q] = (double*)malloc(sizeof(double) * 4 * (scnt[q] > 0 ? scnt[q] : 1));
            gpumpi_parallel_for(nchunk, scatter_chunk, g);
            // the compacted arrays become the species' arrays (with their capacity)
            double* t;
            t = S->x; S->x = S->ax; S->ax = t;
            t = S->y; S->y = S->ay; S->ay = t;
            t = S->u; S->u = S->au; S->au = t;
            t = S->v; S->v = S->av; S->av = t;
            const long tc = S->cap;
            S->cap = S->alt_cap;
            S->alt_cap = tc;
            S->n = stay;
            // counts, then data; the message from neighbour q arrives with tag 100 + (7 - q)
            MPI_Request rq[16];
            double* rbuf[8];
            for (int q = 0; q < 8; q++) {
                MPI_Irecv(&rcnt[q], 1, MPI_INT, nb[q], 100 + (7 - q), MPI_COMM_WORLD, &rq[q]);
                MPI_Isend(&scnt[q], 1, MPI_INT, nb[q], 100 + q, MPI_COMM_WORLD, &rq[8 + q]);
            }
            if (MPI_Waitall(16, rq, MPI_STATUSES_IGNORE) != MPI_SUCCESS) status = 1;
            long nin = 0;
            for (int q = 0; q < 8; q++) {
                rbuf[q] = (double*)malloc(sizeof(double) * 4 * (rcnt[q] > 0 ? rcnt[q] : 1));
                nin += rcnt[q];
                MPI_Irecv(rbuf[q], 4 * rcnt[q], MPI_DOUBLE, nb[q], 200 + (7 - q), MPI_COMM_WORLD, &rq[q]);
                MPI_Isend(g->sbuf[q], 4 * scnt[q], MPI_DOUBLE, nb[q], 200 + q, MPI_COMM_WORLD, &rq[8 + q]);
            }
            if (MPI_Waitall(16, rq, MPI_STATUSES_IGNORE) != MPI_SUCCESS) status = 1;
            if (reserve(S, S->n + nin)) status = 1;
            if (!status) {
                g->roff[0] = 0;
                for (int q = 0; q < 8; q++) {
                    g->rbq[q] = rbuf[q];
                    g->roff[q + 1] = g->roff[q] + rcnt[q];
                }
                g->app_base = S->n;
                gpumpi_parallel_for(nin, append_particle, g);
                S->n += nin;
            }
            for (int q = 0; q < 8; q++) {
                free(g->sbuf[q]);
                free(rbuf[q]);
            }
        }
        // 3. deposit currents (at the new positions), send ghost currents to their owners
        gpumpi_parallel_for(g->cells, clear_current_cell, g);
        gpumpi_parallel_for(nchunk, deposit_chunk, g);
        gpumpi_parallel_for(g->cells, current_from_fixed_cell, g);
        halo_add(g, g->jx, sb, rb, left, right, down, up);
        halo_add(g, g->jy, sb, rb, left, right, down, up);
        // 4. fields: Bz half step from E, E full step from Bz and J, Bz second half step
        halo_fill(g, g->ex, sb, rb, left, right, down, up);
        halo_fill(g, g->ey, sb, rb, left, right, down, up);
        gpumpi_parallel_for(g->ny, bz_half_row, g);
        halo_fill(g, g->bz, sb, rb, left, right, down, up);
        gpumpi_parallel_for(g->ny, e_full_row, g);
        halo_fill(g, g->ex, sb, rb, left, right, down, up);
        halo_fill(g, g->ey, sb, rb, left, right, down, up);
        gpumpi_parallel_for(g->ny, bz_half_row, g);
        // 5. energies
        if (cyc % report == 0 || cyc == cycles) {
            gpumpi_parallel_for(nchunk, energy_chunk, g);
            double ke[NSPEC] = {0.0, 0.0}, e[4], tot[4];
            double fe = 0.0, fb = 0.0;
            for (int c = 0; c < nchunk; c++) {
                ke[0] += g->part[c * 4 + 0];
                ke[1] += g->part[c * 4 + 1];
                fe += g->part[c * 4 + 2];
                fb += g->part[c * 4 + 3];
            }
            e[0] = 0.5 * g->sp[0].mw * ke[0];
            e[1] = 0.5 * g->sp[1].mw * ke[1];
            e[2] = 0.5 * fe;
            e[3] = 0.5 * fb;
            MPI_Allreduce(e, tot, 4, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
            long np = g->sp[0].n + g->sp[1].n, npt = 0;
            MPI_Allreduce(&np, &npt, 1, MPI_LONG, MPI_SUM, MPI_COMM_WORLD);
            if (rank == 0)
                printf("pic cycle %d particles %ld kinetic_e %.17e kinetic_i %.17e electric %.17e magnetic %.17e\n",
                       cyc, npt, tot[0], tot[1], tot[2], tot[3]);
        }
    }
    const double t1 = MPI_Wtime();
    // checksum of every particle's position bits, folded per rank and summed in rank order
    unsigned long long h = 0, hsum = 0;
    for (int s = 0; s < NSPEC; s++)
        for (long k = 0; k < g->sp[s].n; k++) {
            unsigned long long a, b;
            memcpy(&a, &g->sp[s].x[k], 8);
            memcpy(&b, &g->sp[s].y[k], 8);
            h += mix64(a ^ mix64(b));
        }
    MPI_Reduce(&h, &hsum, 1, MPI_UNSIGNED_LONG_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
    double dt_run = t1 - t0, tmax = 0.0;
    MPI_Reduce(&dt_run, &tmax, 1, MPI_DOUBLE, MPI_MAX, 0, MPI_COMM_WORLD);
    int st_all = 0;
    MPI_Allreduce(&status, &st_all, 1, MPI_INT, MPI_MAX, MPI_COMM_WORLD);
    if (rank == 0) {
        printf("pic positions checksum %016llx status %d\n", hsum, st_all);
        printf("pic-time seconds %.6f cycles %d ranks %d (%dx%d)\n", tmax, cycles, size, PX, PY);
    }
    for (int s = 0; s < NSPEC; s++) {
        free(g->sp[s].x);
        free(g->sp[s].y);
        free(g->sp[s].u);
        free(g->sp[s].v);
        free(g->sp[s].ax);
        free(g->sp[s].ay);
        free(g->sp[s].au);
        free(g->sp[s].av);
    }
    free(g->dest);
    free(g->ajx);
    free(g->part);
    free(g->ccount);
    free(g->coff);
    free(fields);
    free(g);
    free(sb);
    free(rb);
    MPI_Finalize();
    return st_all;
}

__device__ int __gpu_max_threads() { return 1024; }
