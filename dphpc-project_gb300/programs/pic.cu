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
// Initial state: PPC particles per cell and species at seeded uniform
// positions, thermal velocities by the Irwin-Hall sum of 12 uniforms (only
// additions, so the host and GPU builds draw identical values), electrons in
// two counter-streaming beams (+-0.1) so that particles migrate.  All
// arithmetic is + - * / on doubles in a fixed order: a GPU run (-fmad=false)
// and a host MPI run give the same bits.
// Rank 0 prints the energies every `report` cycles and a checksum of all
// particle positions at the end.
// Usage: pic [cycles=50] [GX=256] [GY=128] [PPC=125] [report=10]   (P ranks: PX*PY = P, PX >= PY)
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"

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
    double qm;      // charge / mass
    double qw;      // charge of one macro-particle
    double mw;      // mass of one macro-particle
};

// Local grid: (nx+2) x (ny+2) with one ghost layer, index (i+1) + (j+1)*(nx+2).
struct Grid {
    int nx, ny, x0, y0, GX, GY;
    double* ex;
    double* ey;
    double* bz;
    double* jx;
    double* jy;
};

__device__ int gid(const Grid* g, int i, int j) { return (i + 1) + (j + 1) * (g->nx + 2); }

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
__device__ void halo_fill(Grid* g, double* f, double* sb, double* rb, int left, int right, int down, int up) {
    const int nx = g->nx, ny = g->ny, W = nx + 2;
    // x: send my last owned column to the right, receive my left ghost from the left
    for (int j = 0; j < ny; j++) sb[j] = f[gid(g, nx - 1, j)];
    MPI_Sendrecv(sb, ny, MPI_DOUBLE, right, 11, rb, ny, MPI_DOUBLE, left, 11, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int j = 0; j < ny; j++) f[gid(g, -1, j)] = rb[j];
    for (int j = 0; j < ny; j++) sb[j] = f[gid(g, 0, j)];
    MPI_Sendrecv(sb, ny, MPI_DOUBLE, left, 12, rb, ny, MPI_DOUBLE, right, 12, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int j = 0; j < ny; j++) f[gid(g, nx, j)] = rb[j];
    // y: whole rows including the ghost columns
    for (int i = -1; i <= nx; i++) sb[i + 1] = f[gid(g, i, ny - 1)];
    MPI_Sendrecv(sb, W, MPI_DOUBLE, up, 13, rb, W, MPI_DOUBLE, down, 13, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int i = -1; i <= nx; i++) f[gid(g, i, -1)] = rb[i + 1];
    for (int i = -1; i <= nx; i++) sb[i + 1] = f[gid(g, i, 0)];
    MPI_Sendrecv(sb, W, MPI_DOUBLE, down, 14, rb, W, MPI_DOUBLE, up, 14, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    for (int i = -1; i <= nx; i++) f[gid(g, i, ny)] = rb[i + 1];
}

// Add ghost contributions of f to the owners: y rows first (incl. ghost columns), then x columns.
__device__ void halo_add(Grid* g, double* f, double* sb, double* rb, int left, int right, int down, int up) {
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
__device__ void cic(const Grid* g, double px, double py, int* i, int* j, double* fx, double* fy) {
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

__device__ double interp(const Grid* g, const double* f, int i, int j, double fx, double fy) {
    const double a = f[gid(g, i, j)] * (1.0 - fx) + f[gid(g, i + 1, j)] * fx;
    const double b = f[gid(g, i, j + 1)] * (1.0 - fx) + f[gid(g, i + 1, j + 1)] * fx;
    return a * (1.0 - fy) + b * fy;
}

__device__ void deposit(const Grid* g, double* f, int i, int j, double fx, double fy, double val) {
    f[gid(g, i, j)] += val * (1.0 - fx) * (1.0 - fy);
    f[gid(g, i + 1, j)] += val * fx * (1.0 - fy);
    f[gid(g, i, j + 1)] += val * (1.0 - fx) * fy;
    f[gid(g, i + 1, j + 1)] += val * fx * fy;
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
    const int bx = rank % PX, by = rank / PX;
    Grid g;
    g.nx = GX / PX;
    g.ny = GY / PY;
    g.x0 = bx * g.nx;
    g.y0 = by * g.ny;
    g.GX = GX;
    g.GY = GY;
    const int cells = (g.nx + 2) * (g.ny + 2);
    double* fields = (double*)calloc((size_t)cells * 5, sizeof(double));
    g.ex = fields;
    g.ey = fields + cells;
    g.bz = fields + 2 * cells;
    g.jx = fields + 3 * cells;
    g.jy = fields + 4 * cells;
    const int hb = (g.nx > g.ny ? g.nx : g.ny) + 2;
    double* sb = (double*)malloc(sizeof(double) * hb);
    double* rb = (double*)malloc(sizeof(double) * hb);
    const int left = block_rank(bx - 1, by, PX, PY), right = block_rank(bx + 1, by, PX, PY);
    const int down = block_rank(bx, by - 1, PX, PY), up = block_rank(bx, by + 1, PX, PY);
    int nb[8];
    {
        int k = 0;
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++)
                if (dx || dy) nb[k++] = block_rank(bx + dx, by + dy, PX, PY);
    }
    const double dt = 0.5;
    const double uth[NSPEC] = {0.045, 0.009};
    const double qm[NSPEC] = {-1.0, 1.0 / 25.0};
    // plasma frequency 0.1 for electrons: density 1 per cell, w_p^2 = q^2 n / m
    const double qe = 0.1 / (double)PPC;
    Species sp[NSPEC];
    for (int s = 0; s < NSPEC; s++) {
        sp[s].x = sp[s].y = sp[s].u = sp[s].v = nullptr;
        sp[s].n = 0;
        sp[s].cap = 0;
        sp[s].qm = qm[s];
        sp[s].qw = s == 0 ? -qe : qe;
        sp[s].mw = sp[s].qw / sp[s].qm;
        reserve(&sp[s], (long)g.nx * g.ny * PPC + 64);
        unsigned long long seed = mix64(((unsigned long long)rank << 8) + (unsigned long long)s + 1);
        for (int j = 0; j < g.ny; j++)
            for (int i = 0; i < g.nx; i++)
                for (int p = 0; p < PPC; p++) {
                    const long k = sp[s].n++;
                    sp[s].x[k] = (double)(g.x0 + i) + unif(&seed);
                    sp[s].y[k] = (double)(g.y0 + j) + unif(&seed);
                    double a = 0.0, b = 0.0;
                    for (int q = 0; q < 12; q++) a += unif(&seed);
                    for (int q = 0; q < 12; q++) b += unif(&seed);
                    sp[s].u[k] = (a - 6.0) * uth[s] + (s == 0 ? ((p & 1) ? 0.1 : -0.1) : 0.0);
                    sp[s].v[k] = (b - 6.0) * uth[s];
                }
    }
    // migration scratch: counts and per-neighbour index lists
    long* out_idx = nullptr;
    long out_cap = 0;
    MPI_Barrier(MPI_COMM_WORLD);
    const double t0 = MPI_Wtime();
    int status = 0;
    for (int cyc = 1; cyc <= cycles; cyc++) {
        // 1. push and move
        halo_fill(&g, g.ex, sb, rb, left, right, down, up);
        halo_fill(&g, g.ey, sb, rb, left, right, down, up);
        halo_fill(&g, g.bz, sb, rb, left, right, down, up);
        for (int s = 0; s < NSPEC; s++) {
            Species* S = &sp[s];
            const double h = 0.5 * S->qm * dt;
            for (long k = 0; k < S->n; k++) {
                int i, j;
                double fx, fy;
                cic(&g, S->x[k], S->y[k], &i, &j, &fx, &fy);
                const double ex = interp(&g, g.ex, i, j, fx, fy);
                const double ey = interp(&g, g.ey, i, j, fx, fy);
                const double bz = interp(&g, g.bz, i, j, fx, fy);
                // Boris: half kick, rotation about z, half kick
                double um = S->u[k] + h * ex, vm = S->v[k] + h * ey;
                const double t = h * bz;
                const double sfac = 2.0 * t / (1.0 + t * t);
                const double up_ = um + vm * t, vp_ = vm - um * t;
                um = um + vp_ * sfac;
                vm = vm - up_ * sfac;
                S->u[k] = um + h * ex;
                S->v[k] = vm + h * ey;
                double nxp = S->x[k] + S->u[k] * dt, nyp = S->y[k] + S->v[k] * dt;
                if (nxp < 0.0) nxp += (double)GX;
                if (nxp >= (double)GX) nxp -= (double)GX;
                if (nyp < 0.0) nyp += (double)GY;
                if (nyp >= (double)GY) nyp -= (double)GY;
                S->x[k] = nxp;
                S->y[k] = nyp;
            }
        }
        // 2. migrate particles that left the block, species by species
        for (int s = 0; s < NSPEC; s++) {
            Species* S = &sp[s];
            if (S->n > out_cap) {
                free(out_idx);
                out_cap = S->cap;
                out_idx = (long*)malloc(sizeof(long) * out_cap);
            }
            int scnt[8], rcnt[8];
            for (int q = 0; q < 8; q++) scnt[q] = 0;
            long nout = 0;
            // classify: neighbour index 0..7 or -1 (stays)
            for (long k = 0; k < S->n; k++) {
                int cx = (int)S->x[k] / g.nx, cy = (int)S->y[k] / g.ny;
                int dx = cx - bx, dy = cy - by;
                if (dx > 1) dx -= PX;
                if (dx < -1) dx += PX;
                if (dy > 1) dy -= PY;
                if (dy < -1) dy += PY;
                if (dx == 0 && dy == 0) continue;
                int q = (dy + 1) * 3 + (dx + 1);
                if (q > 4) q--;
                out_idx[nout++] = k * 8 + q;
                scnt[q]++;
            }
            // buffers per neighbour: 4 doubles per particle
            double* sbuf[8];
            double* rbuf[8];
            int fill[8];
            for (int q = 0; q < 8; q++) {
                sbuf[q] = (double*)malloc(sizeof(double) * 4 * (scnt[q] > 0 ? scnt[q] : 1));
                fill[q] = 0;
            }
            for (long m = 0; m < nout; m++) {
                const long k = out_idx[m] / 8;
                const int q = (int)(out_idx[m] % 8);
                double* d = sbuf[q] + 4 * fill[q]++;
                d[0] = S->x[k];
                d[1] = S->y[k];
                d[2] = S->u[k];
                d[3] = S->v[k];
            }
            // remove departed particles, keeping the order of the rest
            {
                long w = 0, m = 0;
                for (long k = 0; k < S->n; k++) {
                    if (m < nout && out_idx[m] / 8 == k) {
                        m++;
                        continue;
                    }
                    S->x[w] = S->x[k];
                    S->y[w] = S->y[k];
                    S->u[w] = S->u[k];
                    S->v[w] = S->v[k];
                    w++;
                }
                S->n = w;
            }
            // counts, then data; the message from neighbour q arrives with tag 100 + (7 - q)
            MPI_Request rq[16];
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
                MPI_Isend(sbuf[q], 4 * scnt[q], MPI_DOUBLE, nb[q], 200 + q, MPI_COMM_WORLD, &rq[8 + q]);
            }
            if (MPI_Waitall(16, rq, MPI_STATUSES_IGNORE) != MPI_SUCCESS) status = 1;
            if (reserve(S, S->n + nin)) status = 1;
            for (int q = 0; q < 8 && !status; q++)
                for (int m = 0; m < rcnt[q]; m++) {
                    const double* d = rbuf[q] + 4 * m;
                    const long k = S->n++;
                    S->x[k] = d[0];
                    S->y[k] = d[1];
                    S->u[k] = d[2];
                    S->v[k] = d[3];
                }
            for (int q = 0; q < 8; q++) {
                free(sbuf[q]);
                free(rbuf[q]);
            }
        }
        // 3. deposit currents (at the new positions), send ghost currents to their owners
        for (int c = 0; c < cells; c++) {
            g.jx[c] = 0.0;
            g.jy[c] = 0.0;
        }
        for (int s = 0; s < NSPEC; s++) {
            Species* S = &sp[s];
            for (long k = 0; k < S->n; k++) {
                int i, j;
                double fx, fy;
                cic(&g, S->x[k], S->y[k], &i, &j, &fx, &fy);
                deposit(&g, g.jx, i, j, fx, fy, S->qw * S->u[k]);
                deposit(&g, g.jy, i, j, fx, fy, S->qw * S->v[k]);
            }
        }
        halo_add(&g, g.jx, sb, rb, left, right, down, up);
        halo_add(&g, g.jy, sb, rb, left, right, down, up);
        // 4. fields: Bz half step from E, E full step from Bz and J, Bz second half step
        for (int pass = 0; pass < 2; pass++) {
            halo_fill(&g, g.ex, sb, rb, left, right, down, up);
            halo_fill(&g, g.ey, sb, rb, left, right, down, up);
            for (int j = 0; j < g.ny; j++)
                for (int i = 0; i < g.nx; i++) {
                    const double curl = (g.ey[gid(&g, i + 1, j)] - g.ey[gid(&g, i, j)]) -
                                        (g.ex[gid(&g, i, j + 1)] - g.ex[gid(&g, i, j)]);
                    g.bz[gid(&g, i, j)] -= 0.5 * dt * curl;
                }
            if (pass == 1) break;
            halo_fill(&g, g.bz, sb, rb, left, right, down, up);
            for (int j = 0; j < g.ny; j++)
                for (int i = 0; i < g.nx; i++) {
                    const int c = gid(&g, i, j);
                    g.ex[c] += dt * ((g.bz[c] - g.bz[gid(&g, i, j - 1)]) - g.jx[c]);
                    g.ey[c] += dt * (-(g.bz[c] - g.bz[gid(&g, i - 1, j)]) - g.jy[c]);
                }
        }
        // 5. energies
        if (cyc % report == 0 || cyc == cycles) {
            double e[4] = {0.0, 0.0, 0.0, 0.0}, tot[4];
            for (int s = 0; s < NSPEC; s++) {
                Species* S = &sp[s];
                double ke = 0.0;
                for (long k = 0; k < S->n; k++) ke += S->u[k] * S->u[k] + S->v[k] * S->v[k];
                e[s] = 0.5 * S->mw * ke;
            }
            for (int j = 0; j < g.ny; j++)
                for (int i = 0; i < g.nx; i++) {
                    const int c = gid(&g, i, j);
                    e[2] += g.ex[c] * g.ex[c] + g.ey[c] * g.ey[c];
                    e[3] += g.bz[c] * g.bz[c];
                }
            e[2] *= 0.5;
            e[3] *= 0.5;
            MPI_Allreduce(e, tot, 4, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
            long np = sp[0].n + sp[1].n, npt = 0;
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
        for (long k = 0; k < sp[s].n; k++) {
            unsigned long long a, b;
            memcpy(&a, &sp[s].x[k], 8);
            memcpy(&b, &sp[s].y[k], 8);
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
        free(sp[s].x);
        free(sp[s].y);
        free(sp[s].u);
        free(sp[s].v);
    }
    free(out_idx);
    free(fields);
    free(sb);
    free(rb);
    MPI_Finalize();
    return st_all;
}

__device__ int __gpu_max_threads() { return 1024; }
