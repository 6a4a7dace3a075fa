// Hill-sphere rebinding with every clump's calls on the device (src/tree.hpp:4196-4208).
//
// The reference runs, clump by clump in key order,
//     do { SearchBoundParticlesWithinHillRadius; CalculateHillRadius; } while (it grew)
// where a call that accepts anything ends with SortParticles (src/tree.hpp:4678-4711,
// 4446-4512, 4715-4717). k_rebind_loop runs that whole loop for a clump inside one block:
// a persistent grid (one 512-thread block per SM) takes clumps from a queue in key-rank
// order, so the host is involved once per pass, not once per call. Clumps of one launch run
// concurrently under the ordered-claim rule of the round kernel (owner / tent / defer
// records); a clump may first wait for the lower-ranked clumps it met in the previous pass
// (its blockers). Those were taken from the queue before it by running blocks, so every
// wait ends; each wait is bounded all the same and reports kDevErrLoopLimit if it runs out.
//
// On this GPU an FP64 instruction holds the SM's FP64 pipe for ~19 cycles whatever the
// number of active lanes, and a dependent one waits 36-55 cycles (a division ~590, a square
// root ~630), so the loop keeps FP64 work off its chains:
//  * ball search: the breadth-first frontier of the round kernel, then one block-wide pass
//    over the eligible points of every frontier entry (a contained node keeps all of them,
//    a boundary node keeps those in the ball), compacted in point order;
//  * acceptance: 512 candidates at a time, one per thread in registers (the next 512
//    prefetched meanwhile). Every thread tests its candidate against the current state in
//    FP32 (FP64 when too close to call), the block finds the first bound one, and warp 0
//    applies the reference's FP64 update to the state. Its division is a reciprocal product
//    with Markstein's correction; the reciprocals of the next masses are taken 32 at a time
//    off the dependent chain while the accepted particles have equal masses;
//  * SortParticles: the seven member sums in member order (warp_ordered_sum_window over
//    per-point products m, m x, ..., m vz formed once per snapshot, 128 terms per step with
//    the next terms prefetched into registers), the centre of mass and the Hill radius,
//    squared distances, and a stable sort by squared distance (in shared memory up to
//    kRbSmall members, else a block radix sort on the top 32 bits and an exact fix-up of
//    equal prefixes). Squared distances order members as distances do, except that two
//    squared distances may round to one distance: neighbours within a few ulps are compared
//    through their square roots, and a tie goes to the library-order replay exactly as in
//    the round kernels. The square roots of the last sort are taken when the loop ends.
#pragma once

constexpr int kRB = 512;                      // threads of a rebinding block
constexpr int kRbWarps = kRB / 32;
constexpr uint32_t kRbFront = 4096;           // frontier entries of the ball search
constexpr uint32_t kRbSmall = 4096;           // members sorted in shared memory
constexpr uint32_t kWaitLimit = 1u << 25;     // bounded waits on blockers: sleeps of 1 us per 2^24 points
constexpr uint32_t kCallLimit = 1u << 20;     // calls of one clump in one launch
constexpr int kRbStats = 40;                  // counters per slot
constexpr int kCk = 24;                       // checkpoints per clump and run
// dynamic shared memory: the largest of the frontier, the small sort and the acceptance
// tile (per candidate: FP64 position and velocity, index, FP32 form, taken flag)
constexpr size_t kRbTileBytes = (size_t)kRB * (64 + 4 + sizeof(CandF) + 1);
constexpr size_t kRbSmem14 = 14 * (kRbFront > kRbSmall ? kRbFront : kRbSmall);
constexpr size_t kRbSmem = kRbSmem14 > kRbTileBytes ? kRbSmem14 : kRbTileBytes;
static_assert(kRbFront * 14 <= kRbSmem, "frontier");
static_assert(kRbTileBytes <= kRbSmem, "acceptance tile");
static_assert(kRbSmall * 14 <= kRbSmem, "small sort");
static_assert((256 + 256 * kRbWarps + 1) * 4 <= kRbSmem, "radix counters");

// Checkpoints of the clumps' runs, by key rank: after the calls ck_after() selects, the
// sorted member list (index, squared distance) and the state (M, centre, velocity, Hill
// radius). A rerun resumes from the last checkpoint before its first affected call.
struct Ckpt {
    uint32_t *n;          // per rank: checkpoints kept
    uint32_t *call, *off, *m;  // per rank x kCk: after which call, where in the store, members
    double *st;           // per rank x kCk: M, cx, cy, cz, vx, vy, vz, hill
    uint32_t *idx;        // the store (bump-allocated; a checkpoint that finds it full is not made)
    double *dist;
    uint32_t *top;
    uint32_t cap;
};

// calls 1, 2, 3, 4, 6, 8, 12, 16, 24, 32, ...: a rerun redoes at most a third of the calls
// before its first affected one
__host__ __device__ inline bool ck_after(uint32_t j) {
    if ((j & (j - 1)) == 0) return true;
    return j % 3 == 0 && ((j / 3) & (j / 3 - 1)) == 0;
}

struct RbArgs {
    const uint32_t *list;  // clumps of this launch, in key-rank order
    uint32_t n;
    uint32_t *head;        // next queue position
    const uint32_t *blk_off, *blk;  // blockers of list[i]: blk[blk_off[i], blk_off[i+1]) (slots); null: none
    uint8_t *finished;     // per slot: its calls are done in this launch (or it is not in it)
    uint8_t *suspended;    // per slot: stopped because the member pool is full (state consistent)
    uint8_t *needsort;     // per slot: the last call grew the clump but its SortParticles is pending
    uint8_t *distsq;       // per slot: the segment's distances are still squared
    unsigned long long *stats;  // per slot, kRbStats counters (may be null)
    CT ct;
    Pool P;
    KTree t;
    FTree ft;
    const double4_32a *vel;
    const double4_32a *tm0, *tm1;  // per point: (m, m x, m y, m z), (m vx, m vy, m vz, 0)
    const uint32_t *E, *epos;
    uint32_t *owner;
    const uint32_t *rank_of, *slot_of_rank, *tent;
    uint32_t *dmax, *dset;
    uint8_t *dover;
    const double4_32a *com0;
    unsigned long long *reach;
    CP cp;
    unsigned *err;
    uint32_t wait_limit;   // sleeps a block waits for one blocker before it reports an error
    uint32_t *ccall;       // per slot: calls of the clump's run done (persists across launches)
    uint32_t *dcall, *dfirst;  // per deferral record / per slot: the earliest call that made it
    Ckpt ck;               // ck.n null: no checkpoints
};

// per-point products for the member sums (src/tree.hpp:4436-4440: mass, pos * mass,
// vel * mass, each component rounded once)
__global__ void k_member_terms(uint32_t Tu, const double4_32a *pos, const double4_32a *vel, double4_32a *tm0, double4_32a *tm1) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= Tu) return;
    const double4_32a p = pos[q], v = vel[q];
    tm0[q] = make_double4_32a(p.w, p.x * p.w, p.y * p.w, p.z * p.w);
    tm1[q] = make_double4_32a(v.x * p.w, v.y * p.w, v.z * p.w, 0.0);
}

__device__ __forceinline__ void split_any(double x, float &h, float &l) {
    if (!split_hilo_bits(x, h, l)) split_f(x, h, l);
}

// block-wide compaction offset of this thread's flag; returns the block total
__device__ __forceinline__ uint32_t rb_block_rank(bool keep, uint32_t &rank, uint32_t *warp_tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned b = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_tot[wid] = __popc(b);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < kRbWarps; ++w) {
        const uint32_t c = warp_tot[w];
        if (w < wid) before += c;
        total += c;
    }
    rank = before + __popc(b & ((1u << lane) - 1u));
    __syncthreads();
    return total;
}

// exclusive scan of a[0, n) in shared memory by the whole block; returns the total
__device__ uint32_t rb_scan_excl(uint32_t *a, uint32_t n, uint32_t *warp_tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t per = (n + kRB - 1) / kRB;
    const uint32_t b = threadIdx.x * per, e = min(n, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += a[i];
    uint32_t incl = sum;
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int k = 0; k < kRbWarps; ++k) {
        if (k < wid) before += warp_tot[k];
        total += warp_tot[k];
    }
    uint32_t run = before + incl - sum;
    for (uint32_t i = b; i < e; ++i) {
        const uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
    __syncthreads();
    return total;
}

struct RbShared {
    unsigned char *buf;  // kRbSmem bytes, reused by every phase
    uint32_t *warp_tot;
    uint32_t *u;         // scalars
    double *st;          // M, com x y z, vcom x y z, hill (the call's starting state)
    double *tabM, *tabY; // reciprocal table (warp 0)
    float *tabF;
    float *sf;           // acceptance state for every thread: hi[6], lo[6], Mf
    double *sd;          // acceptance state in FP64: x y z vx vy vz M
};

// ------------------------------------------------------------------ one SearchBound call
// Returns the number of accepted particles, or kNone when the member pool is full (nothing
// changed).
__device__ uint32_t rb_call(const RbArgs &a, uint32_t slot, uint32_t myrank, RbShared &sh, unsigned long long *stat, uint32_t call) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint32_t *front = reinterpret_cast<uint32_t *>(sh.buf), *front2 = front + kRbFront, *fcnt = front2 + kRbFront;
    uint8_t *fcls = reinterpret_cast<uint8_t *>(fcnt + kRbFront), *fcls2 = fcls + kRbFront;
    uint32_t &s_nf = sh.u[0], &s_expand = sh.u[1], &s_noff = sh.u[2], &s_nel = sh.u[3], &s_f = sh.u[4], &s_m0 = sh.u[5],
             &s_o = sh.u[6], &s_S = sh.u[7];
    const long long t0 = clock64();
    if (tid == 0) {
        const double4_32a c = a.ct.com[slot], v = a.ct.vcom[slot];
        sh.st[0] = a.ct.M[slot];
        sh.st[1] = c.x; sh.st[2] = c.y; sh.st[3] = c.z;
        sh.st[4] = v.x; sh.st[5] = v.y; sh.st[6] = v.z;
        sh.st[7] = a.ct.hill[slot];
        s_m0 = a.ct.mn[slot];
        s_o = a.ct.moff[slot];
        front[0] = 0;
        fcls[0] = 0;
        s_nf = 1;
        s_nel = 0;
        const double4_32a c0 = a.com0[slot];  // how far this clump's balls reach from its centre before rebinding
        const double dx = c.x - c0.x, dy = c.y - c0.y, dz = c.z - c0.z;
        const double d = sqrt(dx * dx + dy * dy + dz * dz) + sh.st[7];
        if (d >= 0) atomicMax(&a.reach[slot], (unsigned long long)__double_as_longlong(d));
    }
    __syncthreads();
    const BallQ ball = make_ball(sh.st[1], sh.st[2], sh.st[3], sh.st[7]);
    const KTree &t = a.t;
    // 1) breadth-first frontier (classes 1..4; 0 = not yet classified)
    for (int level = 0; level < 40; ++level) {
        const uint32_t nf = s_nf;
        if (tid == 0) s_expand = 0;
        __syncthreads();
        for (uint32_t i = tid; i < nf; i += kRB) {
            const uint32_t node = front[i];
            int cls = fcls[i];
            if (cls == 0) {
                if (node >= t.nodes) {
                    atomicOr(a.err, (unsigned)kDevErrBadNode);
                    cls = 3;
                } else {
                    uint32_t eb, ee;
                    cls = ball_class(t, a.ft, a.epos, node, ball, eb, ee);
                }
                fcls[i] = (uint8_t)cls;
            }
            fcnt[i] = cls == 4 ? t.nnd[node] : (cls == 3 ? 0u : 1u);
            if (cls == 4) s_expand = 1;
        }
        __syncthreads();
        if (!s_expand) break;
        const uint32_t total = rb_scan_excl(fcnt, nf, sh.warp_tot);
        if (total > kRbFront) break;
        for (uint32_t i = tid; i < nf; i += kRB) {
            const int cls = fcls[i];
            const uint32_t o = fcnt[i];
            if (cls == 1 || cls == 2) {
                front2[o] = front[i];
                fcls2[o] = (uint8_t)cls;
            } else if (cls == 4) {
                const uint32_t c0 = t.nfd[front[i]], nc = t.nnd[front[i]];
                for (uint32_t c = 0; c < nc; ++c) {
                    front2[o + c] = c0 + c;
                    fcls2[o + c] = 0;
                }
            }
        }
        __syncthreads();
        for (uint32_t i = tid; i < total; i += kRB) {
            front[i] = front2[i];
            fcls[i] = fcls2[i];
        }
        if (tid == 0) s_nf = total;
        __syncthreads();
    }
    const uint32_t nf = s_nf;
    // 2) each entry's slice of eligible points: its start (front2) and length (fcnt), scanned
    for (uint32_t i = tid; i < nf; i += kRB) {
        uint32_t eb = 0, ee = 0;
        int cls = fcls[i];
        if (front[i] >= t.nodes) {
            cls = 3;
        } else if (cls == 0) {
            cls = ball_class(t, a.ft, a.epos, front[i], ball, eb, ee);
        } else {
            eb = a.epos[t.nbeg[front[i]]];
            ee = a.epos[t.nend[front[i]]];
        }
        fcls[i] = (uint8_t)cls;
        front2[i] = eb;
        fcnt[i] = cls == 3 ? 0u : ee - eb;
    }
    __syncthreads();
    const uint32_t S = rb_scan_excl(fcnt, nf, sh.warp_tot);
    // 3) the new segment: the members, then room for every scanned point
    if (tid == 0) {
        s_S = S;
        s_noff = pool_try_alloc(a.P, s_m0 + S);
    }
    __syncthreads();
    if (s_noff == kNone) return kNone;
    const uint32_t m0 = s_m0, o = s_o, no = s_noff;
    for (uint32_t k = tid; k < m0; k += kRB) a.P.idx[no + k] = a.P.idx[o + k];
    uint32_t *elig = a.P.idx + no + m0;
    for (uint32_t base = 0; base < S; base += kRB) {
        const uint32_t tt = base + tid;
        bool keep = false;
        uint32_t q = 0;
        if (tt < S) {
            uint32_t lo = 0, hi = nf;  // the last entry starting at or before tt
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (fcnt[mid] <= tt) lo = mid;
                else hi = mid;
            }
            q = a.E[front2[lo] + (tt - fcnt[lo])];
            keep = fcls[lo] == 1 || in_ball(t, a.ft, ball, q);
            // this clump's own claims are its members: the acceptance would only skip them
            if (keep && __ldcg(&a.owner[q]) == myrank) keep = false;
        }
        uint32_t r;
        const uint32_t tot = rb_block_rank(keep, r, sh.warp_tot);
        if (keep) elig[s_nel + r] = q;
        __syncthreads();
        if (tid == 0) s_nel += tot;
        __syncthreads();
    }
    const uint32_t nel = s_nel;
    const long long t1 = clock64();
    // 4) the reference's sequential acceptance (src/tree.hpp:4686-4706), 512 candidates at a
    // time. Every thread holds one candidate (its FP32 form in registers; the FP64 position
    // and velocity, the index, the FP32 form and the taken flag also in shared memory). The
    // block finds the first bound candidate; warp 0 takes it and then goes on alone through
    // the next candidates, 32 at a time, as long as each 32 holds a bound one (no block
    // barrier per acceptance where acceptances are dense); the block search resumes after a
    // 32 without any.
    double4_32a *tpos = reinterpret_cast<double4_32a *>(sh.buf), *tvel = tpos + kRB;
    uint32_t *tq = reinterpret_cast<uint32_t *>(tvel + kRB);
    CandF *tf = reinterpret_cast<CandF *>(tq + kRB);
    uint8_t *ttk = reinterpret_cast<uint8_t *>(tf + kRB);
    uint32_t &s_pos = sh.u[8];
    const float G32 = (float)a.cp.G, shear32 = (float)a.cp.shear;
    double comp = 0.0;      // warp 0, lane c < 6: component c of the state (x y z vx vy vz)
    double M = sh.st[0];    // warp 0: the mass
    double tab_m = -1.0;    // warp 0: the mass the reciprocal table was built for
    int tab_n = 0, tab_i = 0;
    uint32_t nacc = 0, rounds = 0;
    if (tid == 0) {
        sh.u[12] = 0;
        sh.u[13] = 0;
        sh.u[14] = 0;
        sh.u[15] = 0;
        sh.u[16] = 0;
        sh.u[17] = 0;
        sh.u[18] = 0;
    }
    if (tid < 32) {
        comp = lane < 6 ? sh.st[1 + lane] : 0.0;
        float h = 0.f, l = 0.f;
        split_any(comp, h, l);
        if (lane < 6) {
            sh.sf[lane] = h;
            sh.sf[6 + lane] = l;
            sh.sd[lane] = comp;
        }
        if (lane == 0) {
            float mh, ml;
            split_any(M, mh, ml);
            sh.sf[12] = mh;
            sh.sd[6] = M;
        }
    }
    // warp 0 takes candidate j of the tile: the reference's update (src/tree.hpp:4696-4701,
    // the new mass multiplies the old centre), lane c < 6 updating component c as
    // RN(RN(RN(c M') + RN(m q_c)) / M'); the new state is published in shared memory
    auto take = [&](uint32_t j) {
        const unsigned full = 0xffffffffu;
        const long long tu0 = clock64();
        const double m = tpos[j].w;
        if (!(tab_i < tab_n && dbits(m) == dbits(tab_m))) {
            // the next masses M_{l+1} = RN(M_l + m) on the grid of M's binade (exact while
            // they stay inside it), and their correctly rounded reciprocals
            tab_m = m;
            tab_i = 0;
            tab_n = 0;
            const uint64_t mb = dbits(M);
            const uint32_t ex = (uint32_t)(mb >> 52) & 0x7ffu;
            long long dn = 0;
            if ((mb >> 63) == 0 && ex > 60u && ex < 2000u && grid_term(m, ex, dn) && dn > 0) {
                const long long n0 = (long long)((mb & 0xfffffffffffffull) | (1ull << 52));
                const long long nl = n0 + (long long)(lane + 1) * dn;
                const bool ok = nl > (1LL << 52) && nl <= (1LL << 53);
                const unsigned okm = __ballot_sync(full, ok);
                const unsigned edge = __ballot_sync(full, ok && nl == (1LL << 53));
                int cnt = (~okm) ? __ffs(~okm) - 1 : 32;
                if (edge) cnt = min(cnt, __ffs(edge));
                if (lane < cnt) {
                    const double Ml = grid_value(nl, ex);
                    float fh, fl;
                    split_any(Ml, fh, fl);
                    sh.tabM[lane] = Ml;
                    sh.tabY[lane] = __drcp_rn(Ml);
                    sh.tabF[lane] = fh;
                }
                tab_n = cnt;
                __syncwarp();
            }
        }
        const long long tu1 = clock64();
        double Mn, y;
        float Mnf;
        if (tab_i < tab_n) {
            Mn = sh.tabM[tab_i];
            y = sh.tabY[tab_i];
            Mnf = sh.tabF[tab_i];
            ++tab_i;
        } else {
            Mn = M + m;
            y = __drcp_rn(Mn);
            float fl;
            split_any(Mn, Mnf, fl);
            tab_n = 0;
        }
        if (lane < 6) {
            // each lane loads its own component (one shared-memory load; a select over the
            // whole position and velocity costs several hundred cycles here)
            const double qc = reinterpret_cast<const double *>(lane < 3 ? &tpos[j] : &tvel[j])[lane < 3 ? lane : lane - 3];
            const double num = comp * Mn + m * qc;
            if ((dbits(num) << 1) == 0) {
                comp = num;  // the quotient keeps the numerator's zero
            } else {
                const double q0 = num * y;
                comp = fma(fma(-q0, Mn, num), y, q0);
            }
            float h, l;
            if (stat && lane == 0) sh.u[15] += (uint32_t)(clock64() - tu1);
            split_f(comp, h, l);  // the FP64 pipe is idle here: its conversions beat the integer split
            sh.sf[lane] = h;
            sh.sf[6 + lane] = l;
            sh.sd[lane] = comp;
        }
        M = Mn;
        if (lane == 0) {
            sh.sf[12] = Mnf;
            sh.sd[6] = Mn;
            const uint32_t q2 = tq[j];
            // the lowest rank keeps the particle; who lost one is found after the pass
            atomicMin(&a.owner[q2], myrank);
            elig[nacc] = q2;  // accepted ones overwrite candidates already consumed
            if (stat) {
                sh.u[13] += (uint32_t)(clock64() - tu0);
                sh.u[14] += (uint32_t)(tu1 - tu0);
            }
        }
        ++nacc;
        __syncwarp();
    };
    // the prefetched candidate of the next tile
    uint32_t nq = kNone, now_ = kNone, ntn = kNone;
    double4_32a np = make_double4_32a(0, 0, 0, 0), nv = make_double4_32a(0, 0, 0, 0);
    float4 nph = make_float4(0.f, 0.f, 0.f, 0.f), npl = nph;
    if ((uint32_t)tid < nel) {
        nq = elig[tid];
        now_ = __ldcg(&a.owner[nq]);
        ntn = a.tent[nq];
        np = t.pos[nq];
        nv = a.vel[nq];
        nph = a.ft.phi[nq];
        npl = a.ft.plo[nq];
    }
    long long t_setup = 0;
    uint32_t n_tiles = 0;
    for (uint32_t base = 0; base < nel; base += kRB) {
        const long long tt0 = clock64();
        const uint32_t q = nq;
        const uint32_t tlen = min((uint32_t)kRB, nel - base);
        const bool valid = q != kNone;
        bool taken = true;
        CandF cf;
        if (valid) {
            uint32_t ow = now_, tn = ntn;
            if (tn != kNone && tn < myrank && *(volatile const uint8_t *)&a.finished[a.slot_of_rank[tn]]) {
                // that clump has finished its calls in this launch: its claims are its
                // holdings, and its prediction from the last pass no longer applies
                __threadfence();
                ow = __ldcg(&a.owner[q]);
                tn = kNone;
            }
            taken = (ow != kNone && ow <= myrank) || (tn != kNone && tn < myrank);
            if (stat) {
                if (tn != kNone && tn < myrank) atomicAdd(&sh.u[16], 1u);
                if (ow != kNone && ow < myrank) atomicAdd(&sh.u[17], 1u);
                if (taken) atomicAdd(&sh.u[18], 1u);
            }
            if (ow != kNone && ow < myrank)
                defer_add(a.dset, a.dover, a.dmax, slot, ow, *(volatile const uint8_t *)&a.finished[a.slot_of_rank[ow]] == 0, a.dcall,
                          a.dfirst, call);
            else if (tn != kNone && tn < myrank)
                defer_add(a.dset, a.dover, a.dmax, slot, tn, true, a.dcall, a.dfirst, call);
            tpos[tid] = np;
            tvel[tid] = nv;
            tq[tid] = q;
            cf.ph[0] = nph.x; cf.ph[1] = nph.y; cf.ph[2] = nph.z;
            cf.pl[0] = npl.x; cf.pl[1] = npl.y; cf.pl[2] = npl.z;
            split_any(nv.x, cf.vh[0], cf.vl[0]);
            split_any(nv.y, cf.vh[1], cf.vl[1]);
            split_any(nv.z, cf.vh[2], cf.vl[2]);
            float wl;
            split_any(np.w, cf.w, wl);
            tf[tid] = cf;
        }
        ttk[tid] = taken ? 1 : 0;
        nq = kNone;
        if (base + kRB + tid < nel) {  // prefetch (accepted ones are written below base + kRB only)
            nq = elig[base + kRB + tid];
            now_ = __ldcg(&a.owner[nq]);
            ntn = a.tent[nq];
            np = t.pos[nq];
            nv = a.vel[nq];
            nph = a.ft.phi[nq];
            npl = a.ft.plo[nq];
        }
        __syncthreads();
        t_setup += clock64() - tt0;
        ++n_tiles;
        for (uint32_t pos = 0;;) {
            ++rounds;
            bool bound = false, unsure = false;
            if (valid && !taken && (uint32_t)tid >= pos) {
                float shv[6], slv[6];
                for (int c = 0; c < 6; ++c) {
                    shv[c] = sh.sf[c];
                    slv[c] = sh.sf[6 + c];
                }
                const int r = bound_hilo_fast(cf, sh.sf[12], shv, slv, G32, shear32);
                if (r >= 0) bound = r == 1;
                else unsure = true;
            }
            if (unsure) {
                bound = bound_fp64(tpos[tid], tvel[tid], sh.sd[6], sh.sd[0], sh.sd[1], sh.sd[2], sh.sd[3], sh.sd[4], sh.sd[5], a.cp);
                if (stat) atomicAdd(&sh.u[12], 1u);
            }
            const unsigned b = __ballot_sync(0xffffffffu, bound);
            if (lane == 0) sh.warp_tot[wid] = b ? (uint32_t)(wid * 32 + __ffs(b) - 1) : kNone;
            __syncthreads();
            uint32_t f = kNone;
            {
                uint32_t wv[kRbWarps];
                for (int w = 0; w < kRbWarps; ++w) wv[w] = sh.warp_tot[w];
                for (int w = kRbWarps - 1; w >= 0; --w) f = wv[w] != kNone ? wv[w] : f;
            }
            if (f == kNone) break;  // the rest of the tile is not bound
            if (tid < 32) {
                const unsigned full = 0xffffffffu;
                take(f);
                // warp 0 alone through the next candidates while acceptances are dense
                uint32_t at = f + 1;
                while (at < tlen) {
                    const uint32_t k = at + lane;
                    bool bd = false, un = false;
                    if (k < tlen && !ttk[k]) {
                        float shv[6], slv[6];
                        for (int c = 0; c < 6; ++c) {
                            shv[c] = sh.sf[c];
                            slv[c] = sh.sf[6 + c];
                        }
                        const int r = bound_hilo_fast(tf[k], sh.sf[12], shv, slv, G32, shear32);
                        if (r >= 0) bd = r == 1;
                        else un = true;
                    }
                    if (un) {
                        bd = bound_fp64(tpos[k], tvel[k], sh.sd[6], sh.sd[0], sh.sd[1], sh.sd[2], sh.sd[3], sh.sd[4], sh.sd[5], a.cp);
                        if (stat) atomicAdd(&sh.u[12], 1u);
                    }
                    const unsigned bb = __ballot_sync(full, bd);
                    if (!bb) {  // none of these 32 is bound: leave them, back to the block search
                        at = min(at + 32u, tlen);
                        break;
                    }
                    const uint32_t j = at + (uint32_t)(__ffs(bb) - 1);
                    take(j);
                    at = j + 1;
                }
                if (lane == 0) s_pos = at;
            }
            __syncthreads();
            pos = s_pos;
            if (pos >= tlen) break;
        }
        __syncthreads();
    }
    if (tid == 0) s_f = nacc;
    __syncthreads();
    nacc = s_f;
    const long long t2 = clock64();
    if (tid == 0) {
        if (stat) {
            stat[0] += 1;
            stat[1] += nel;
            stat[2] += nacc;
            stat[3] += (unsigned long long)(t1 - t0);
            stat[4] += (unsigned long long)(t2 - t1);
            stat[12] += rounds;
            stat[13] += S;
            stat[10] += sh.u[12];
            stat[14] += sh.u[13];
            stat[15] += sh.u[14];  // of which the table look-up / rebuild
            stat[16] += sh.u[15];  // and the FP64 update chain
            stat[31] += (unsigned long long)t_setup;  // tile set-up: loads arriving, filters, splits
            stat[32] += n_tiles;
            stat[33] += sh.u[16];  // candidates predicted for an earlier clump
            stat[34] += sh.u[17];  // held by an earlier clump
            stat[35] += sh.u[18];  // taken either way
        }
        if (nacc) {
            a.ct.moff[slot] = no;
            a.ct.mn[slot] = m0 + nacc;
        } else {
            atomicCAS(a.P.top, no + m0 + S, no);  // give the segment back when nothing was taken after it
        }
    }
    __syncthreads();
    return nacc;
}

// ------------------------------------------------------------------ SortParticles
// Block radix sort (stable, 8-bit digits) of n (key, value) pairs from (ki, vi) into the
// other buffer pair; digits that are the same for every key are skipped. Returns 0 when
// the result is in (ki, vi), 1 when in (ko, vo).
__device__ int rb_radix32(uint32_t *ki, uint32_t *vi, uint32_t *ko, uint32_t *vo, uint32_t n, uint32_t *smem) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint32_t *hist = smem, *wcnt = smem + 256, *flag = smem + 256 + 256 * kRbWarps;
    int where = 0;
    for (int pass = 0; pass < 4; ++pass) {
        const int sh = 8 * pass;
        uint32_t *kin = where ? ko : ki, *vin = where ? vo : vi, *kout = where ? ki : ko, *vout = where ? vi : vo;
        for (int d = tid; d < 256; d += kRB) hist[d] = 0;
        for (int d = tid; d < 256 * kRbWarps; d += kRB) wcnt[d] = 0;
        if (tid == 0) flag[0] = 0;
        __syncthreads();
        for (uint32_t i = tid; i < n; i += kRB) atomicAdd(&hist[(kin[i] >> sh) & 255u], 1u);
        __syncthreads();
        for (int d = tid; d < 256; d += kRB)
            if (hist[d] == n) flag[0] = 1;
        __syncthreads();
        if (flag[0]) continue;  // every key has this digit
        if (tid < 32) {  // exclusive scan of the 256 bins by warp 0, 8 per lane
            uint32_t v[8], s = 0;
            for (int q = 0; q < 8; ++q) { v[q] = hist[lane * 8 + q]; s += v[q]; }
            uint32_t incl = s;
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += u;
            }
            uint32_t run = incl - s;
            for (int q = 0; q < 8; ++q) { hist[lane * 8 + q] = run; run += v[q]; }
        }
        __syncthreads();
        for (uint32_t b = 0; b < n; b += kRB) {
            const uint32_t i = b + tid;
            const bool valid = i < n;
            const uint32_t key = valid ? kin[i] : 0u, val = valid ? vin[i] : 0u;
            const uint32_t dig = valid ? (key >> sh) & 255u : 256u;
            const unsigned peers = __match_any_sync(0xffffffffu, dig);
            const uint32_t rk = __popc(peers & ((1u << lane) - 1u));
            if (valid && (uint32_t)(__ffs(peers) - 1) == (uint32_t)lane) wcnt[wid * 256 + dig] = __popc(peers);
            __syncthreads();
            if (valid) {
                uint32_t off = hist[dig];
                for (int w = 0; w < wid; ++w) off += wcnt[w * 256 + dig];
                kout[off + rk] = key;
                vout[off + rk] = val;
            }
            __syncthreads();
            for (int d = tid; d < 256; d += kRB) {
                uint32_t tot = 0;
                for (int w = 0; w < kRbWarps; ++w) {
                    tot += wcnt[w * 256 + d];
                    wcnt[w * 256 + d] = 0;
                }
                hist[d] += tot;
            }
            __syncthreads();
        }
        where ^= 1;
    }
    return where;
}

// any two neighbours of a sorted run of squared distances whose square roots are equal
__device__ __forceinline__ bool rb_sqrt_tie(double s0, double s1) {
    if (s0 == s1) return true;
    const unsigned long long b0 = (unsigned long long)__double_as_longlong(s0), b1 = (unsigned long long)__double_as_longlong(s1);
    if (b1 - b0 > 64ull) return false;  // more than a few ulps apart: the roots differ
    return sqrt(s0) == sqrt(s1);
}

// SortParticles with the Hill radius after it (src/tree.hpp:4446-4512, 4715-4717). Returns
// false when the pool has no room for a large sort (the clump is then left with needsort).
__device__ bool rb_sort_particles(const RbArgs &a, uint32_t slot, RbShared &sh, unsigned long long *stat) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint32_t &s_o = sh.u[8], &s_m = sh.u[9], &s_tie = sh.u[10], &s_r = sh.u[11];
    const long long t0 = clock64();
    if (tid == 0) {
        s_o = a.ct.moff[slot];
        s_m = a.ct.mn[slot];
        s_tie = 0;
    }
    __syncthreads();
    const uint32_t o = s_o, m = s_m;
    uint32_t *idx = a.P.idx + o;
    double *dist = a.P.dist + o;
    // 1) the seven sums in member order (CalculateKinematicProperties): warp w < 7 runs sum w
    // over the per-point products, 64 terms per step, from a shared-memory stage that the
    // other nine warps fill: 256 members at a time (one per loading thread), double-buffered,
    // the member indices of a chunk read one chunk ahead, so the sums never wait on a gather
    // from memory
    double acc = 0.0;
    uint32_t its = 0;
    long long tsum = 0;
    {
        constexpr uint32_t kCh = 256;            // members per chunk
        constexpr uint32_t kLd = kRB - 7 * 32;   // loading threads (warps 7..15)
        constexpr int kK = 2;                    // terms per lane and step
        static_assert(2 * 7 * kCh * sizeof(double) <= kRbSmem, "sum stage");
        static_assert(kCh <= kLd && kCh % (32 * kK) == 0, "sum chunk");
        double *stg = reinterpret_cast<double *>(sh.buf);  // [2][7][kCh]
        auto put = [&](double *d, uint32_t k, const double4_32a &p, const double4_32a &v) {
            d[k] = p.x;
            d[kCh + k] = p.y;
            d[2 * kCh + k] = p.z;
            d[3 * kCh + k] = p.w;
            d[4 * kCh + k] = v.x;
            d[5 * kCh + k] = v.y;
            d[6 * kCh + k] = v.z;
        };
        const uint32_t nch = (m + kCh - 1) / kCh;
        if ((uint32_t)tid < min(m, kCh)) {  // chunk 0: every thread
            const uint32_t q = idx[tid];
            put(stg, (uint32_t)tid, a.tm0[q], a.tm1[q]);
        }
        const uint32_t k0 = (uint32_t)tid - 7u * 32u;  // loading threads: their member of a chunk
        uint32_t q0 = 0;                              // and its index in the next chunk
        if (wid >= 7 && k0 < kCh && kCh + k0 < m) q0 = idx[kCh + k0];
        __syncthreads();
        const long long ts = clock64();
        for (uint32_t c = 0; c < nch; ++c) {
            const uint32_t b = c & 1u;
            if (wid < 7) {
                const double *src = stg + ((size_t)b * 7 + wid) * kCh;
                const uint32_t cnt = min(kCh, m - c * kCh);
                for (uint32_t w0 = 0; w0 < cnt; w0 += 32 * kK) {
                    const uint32_t k = w0 + (uint32_t)lane * kK;
                    double x[kK];
                    const double2 v2 = k < cnt ? *reinterpret_cast<const double2 *>(src + k) : make_double2(0.0, 0.0);
                    x[0] = v2.x;
                    x[1] = k + 1 < cnt ? v2.y : 0.0;
                    acc = warp_ordered_sum_window<kK>(x, min(32u * kK, cnt - w0), acc, &its);
                }
            } else if (c + 1 < nch && k0 < kCh) {
                // chunk c + 1 into the other buffer, and the index of chunk c + 2
                const uint32_t g1 = (c + 1) * kCh, g2 = g1 + kCh;
                if (g1 + k0 < m) {
                    const double4_32a p0 = a.tm0[q0], u0 = a.tm1[q0];
                    q0 = g2 + k0 < m ? idx[g2 + k0] : 0u;
                    put(stg + (size_t)(b ^ 1u) * 7 * kCh, k0, p0, u0);
                }
            }
            __syncthreads();
        }
        tsum = clock64() - ts;
    }
    if (wid < 7 && lane == 0) sh.tabM[wid] = acc;  // the table is free between calls
    if (wid < 7 && lane == 0 && stat) {  // each sum: its time and its steps
        atomicAdd(&stat[17 + wid], (unsigned long long)its);
        atomicAdd(&stat[24 + wid], (unsigned long long)tsum);
    }
    __syncthreads();
    if (tid < 32) {
        const double Ms = sh.tabM[0];
        double v = 0.0;
        if (lane >= 1 && lane <= 6) v = sh.tabM[lane] / Ms;
        if (lane == 7) v = cr_pow_third(Ms * a.cp.G / 3. / a.cp.Omega / a.cp.Omega);  // src/tree.hpp:4715-4717
        if (lane >= 1 && lane <= 7) sh.st[lane] = v;
        if (lane == 0) sh.st[0] = Ms;
    }
    __syncthreads();
    const long long t_sum = clock64();
    if (tid == 0) {
        a.ct.M[slot] = sh.st[0];
        a.ct.com[slot] = make_double4_32a(sh.st[1], sh.st[2], sh.st[3], 0);
        a.ct.vcom[slot] = make_double4_32a(sh.st[4], sh.st[5], sh.st[6], 0);
        a.ct.hill[slot] = sh.st[7];
    }
    // 2) squared distances to the new centre (src/tree.hpp:4448-4450: (pos - com).Norm())
    const double cx = sh.st[1], cy = sh.st[2], cz = sh.st[3];
    for (uint32_t k = tid; k < m; k += kRB) {
        const double4_32a p = a.t.pos[idx[k]];
        const double dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
        double s = dx * dx;
        s = s + dy * dy;
        s = s + dz * dz;
        dist[k] = s;
    }
    __syncthreads();
    const long long t_dist = clock64();
    bool ok = true;
    if (m <= kRbSmall) {
        // 3a) in shared memory: bitonic sort by (squared distance, position)
        unsigned long long *sk = reinterpret_cast<unsigned long long *>(sh.buf);
        uint32_t *si = reinterpret_cast<uint32_t *>(sk + kRbSmall);
        uint16_t *sp = reinterpret_cast<uint16_t *>(si + kRbSmall);
        uint32_t n2 = 1;
        while (n2 < m) n2 <<= 1;
        for (uint32_t k = tid; k < n2; k += kRB) {
            if (k < m) {
                sk[k] = (unsigned long long)__double_as_longlong(dist[k]);
                si[k] = idx[k];
                sp[k] = (uint16_t)k;
            } else {
                sk[k] = ~0ull;
                si[k] = kNone;
                sp[k] = 0xffff;
            }
        }
        __syncthreads();
        for (uint32_t size = 2; size <= n2; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (uint32_t k = tid; k < n2; k += kRB) {
                    const uint32_t j = k ^ stride;
                    if (j > k) {
                        const bool up = (k & size) == 0;
                        const bool gt = sk[k] > sk[j] || (sk[k] == sk[j] && sp[k] > sp[j]);
                        if (gt == up) {
                            const unsigned long long tk = sk[k]; sk[k] = sk[j]; sk[j] = tk;
                            const uint32_t ti = si[k]; si[k] = si[j]; si[j] = ti;
                            const uint16_t tp = sp[k]; sp[k] = sp[j]; sp[j] = tp;
                        }
                    }
                }
                __syncthreads();
            }
        }
        // (every size: below 17 members the library's insertion sort is stable by distance,
        // which an order by squared distance only equals when no two roots tie)
        int tie = 0;
        for (uint32_t k = tid + 1; k < m; k += kRB)
            tie |= rb_sqrt_tie(__longlong_as_double((long long)sk[k - 1]), __longlong_as_double((long long)sk[k]));
        if (__syncthreads_or(tie)) {
            if (tid == 0) s_tie = 1;
        } else {
            for (uint32_t k = tid; k < m; k += kRB) {
                idx[k] = si[k];
                dist[k] = __longlong_as_double((long long)sk[k]);
            }
        }
        __syncthreads();
    } else {
        // 3b) large: radix sort of the top 32 bits with the position as payload into three
        // fresh pool areas (D: the sorted segment; X, Y: sort buffers, given back after)
        if (tid == 0) s_r = pool_try_alloc(a.P, 3 * m);
        __syncthreads();
        const uint32_t r = s_r;
        if (r == kNone) {
            ok = false;
        } else {
            uint32_t *kx = a.P.idx + r + m, *ky = a.P.idx + r + 2 * m;
            uint32_t *vx = reinterpret_cast<uint32_t *>(a.P.dist + r + m), *vy = reinterpret_cast<uint32_t *>(a.P.dist + r + 2 * m);
            for (uint32_t k = tid; k < m; k += kRB) {
                kx[k] = (uint32_t)((unsigned long long)__double_as_longlong(dist[k]) >> 32);
                vx[k] = k;
            }
            __syncthreads();
            const int where = rb_radix32(kx, vx, ky, vy, m, reinterpret_cast<uint32_t *>(sh.buf));
            const uint32_t *ks = where ? ky : kx, *vs = where ? vy : vx;
            uint32_t *didx = a.P.idx + r;
            double *ddist = a.P.dist + r;
            for (uint32_t k = tid; k < m; k += kRB) {
                const uint32_t src = vs[k];
                didx[k] = idx[src];
                ddist[k] = dist[src];
            }
            __syncthreads();
            // runs of equal top bits: insertion sort by the full squared distance (stable)
            for (uint32_t k = tid; k < m; k += kRB) {
                if ((k == 0 || ks[k] != ks[k - 1]) && k + 1 < m && ks[k + 1] == ks[k]) {
                    uint32_t e = k + 1;
                    while (e < m && ks[e] == ks[k]) ++e;
                    for (uint32_t i = k + 1; i < e; ++i) {
                        const double dv = ddist[i];
                        const uint32_t iv = didx[i];
                        uint32_t j = i;
                        while (j > k && ddist[j - 1] > dv) {
                            ddist[j] = ddist[j - 1];
                            didx[j] = didx[j - 1];
                            --j;
                        }
                        ddist[j] = dv;
                        didx[j] = iv;
                    }
                }
            }
            __syncthreads();
            int tie = 0;
            for (uint32_t k = tid + 1; k < m; k += kRB) tie |= rb_sqrt_tie(ddist[k - 1], ddist[k]);
            if (__syncthreads_or(tie)) {
                if (tid == 0) s_tie = 1;  // the unsorted segment at o is intact
            } else if (tid == 0) {
                a.ct.moff[slot] = r;
            }
            if (tid == 0) atomicCAS(a.P.top, r + 3 * m, r + m);  // give X and Y back when they are on top
            __syncthreads();
        }
    }
    if (ok && s_tie) {
        // two members at the same distance: the library's std::sort order on the sequence
        // before the sort, with the distances themselves (lib_sort.cuh, one thread)
        for (uint32_t k = tid; k < m; k += kRB) dist[k] = sqrt(dist[k]);
        __syncthreads();
        if (tid == 0) lib_sort(dist, idx, m);
        __syncthreads();
    }
    if (tid == 0) {
        if (ok) {
            a.needsort[slot] = 0;
            a.distsq[slot] = s_tie ? 0 : 1;
        } else {
            a.needsort[slot] = 1;
        }
        if (stat) {
            const long long t3 = clock64();
            stat[5] += (unsigned long long)(t3 - t0);
            stat[6] += (unsigned long long)(t_sum - t0);
            stat[7] += 1;
            stat[8] += (unsigned long long)(t_dist - t_sum);
            stat[9] += (unsigned long long)(t3 - t_dist);
            stat[11] += m;
        }
    }
    __syncthreads();
    return ok;
}

// ------------------------------------------------------------------ checkpoints
__device__ uint32_t ck_try_alloc(const Ckpt &ck, uint32_t n) {
    uint32_t cur = *(volatile uint32_t *)ck.top;
    for (int it = 0; it < (1 << 22); ++it) {
        if ((uint64_t)cur + n > ck.cap) return kNone;
        const uint32_t prev = atomicCAS(ck.top, cur, cur + n);
        if (prev == cur) return cur;
        cur = prev;
    }
    return kNone;
}

// the clump's state after call j (its members just sorted): a checkpoint, if there is room
__device__ void rb_checkpoint(const RbArgs &a, uint32_t slot, uint32_t rank, uint32_t j, RbShared &sh) {
    const int tid = threadIdx.x;
    uint32_t &s_off = sh.u[19];
    const uint32_t o = a.ct.moff[slot], m = a.ct.mn[slot];
    if (tid == 0) {
        s_off = kNone;
        if (a.ck.n[rank] < (uint32_t)kCk) s_off = ck_try_alloc(a.ck, m);
    }
    __syncthreads();
    const uint32_t off = s_off;
    if (off != kNone) {
        for (uint32_t k = tid; k < m; k += kRB) {
            a.ck.idx[off + k] = a.P.idx[o + k];
            a.ck.dist[off + k] = a.P.dist[o + k];
        }
        if (tid == 0) {
            const uint32_t n = a.ck.n[rank];
            const size_t e = (size_t)rank * kCk + n;
            const double4_32a c = a.ct.com[slot], v = a.ct.vcom[slot];
            double *q = a.ck.st + e * 8;
            q[0] = a.ct.M[slot];
            q[1] = c.x; q[2] = c.y; q[3] = c.z;
            q[4] = v.x; q[5] = v.y; q[6] = v.z;
            q[7] = a.ct.hill[slot];
            a.ck.call[e] = j;
            a.ck.off[e] = off;
            a.ck.m[e] = m;
            a.ck.n[rank] = n + 1;
        }
    }
    __syncthreads();
}

// ------------------------------------------------------------------ the persistent loop
__global__ void __launch_bounds__(kRB, 1) k_rebind_loop(RbArgs a) {
    extern __shared__ __align__(16) unsigned char rb_dyn[];
    __shared__ uint32_t warp_tot[kRbWarps];
    __shared__ uint32_t u[20];
    __shared__ double st[8], tabM[32], tabY[32], sd[8];
    __shared__ float tabF[32], sf[16];
    __shared__ uint32_t s_item;
    RbShared sh{rb_dyn, warp_tot, u, st, tabM, tabY, tabF, sf, sd};
    const int tid = threadIdx.x;
    for (uint32_t guard = 0; guard <= a.n; ++guard) {
        if (tid == 0) s_item = atomicAdd(a.head, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        __syncthreads();
        if (item >= a.n) return;
        const uint32_t slot = a.list[item];
        if (tid == 0 && a.blk_off) {
            for (uint32_t b = a.blk_off[item]; b < a.blk_off[item + 1]; ++b) {
                const uint32_t bs = a.blk[b];
                for (uint32_t it = 0; *(volatile uint8_t *)&a.finished[bs] == 0; ++it) {
                    if (it >= a.wait_limit) {
                        atomicOr(a.err, (unsigned)kDevErrLoopLimit);
                        break;
                    }
                    __nanosleep(1000);
                }
            }
            __threadfence();
        }
        __syncthreads();
        const uint32_t myrank = a.rank_of[slot];
        unsigned long long *stat = a.stats ? a.stats + kRbStats * (size_t)slot : nullptr;
        if (tid == 0) s_item = a.ccall ? a.ccall[slot] : 0u;
        __syncthreads();
        uint32_t done = s_item;  // calls of this clump's run so far
        __syncthreads();
        bool suspend = false;
        if (a.needsort[slot]) suspend = !rb_sort_particles(a, slot, sh, stat);
        for (uint32_t call = 0; !suspend; ++call) {
            if (call >= kCallLimit) {
                if (tid == 0) atomicOr(a.err, (unsigned)kDevErrLoopLimit);
                break;
            }
            const uint32_t j = done + 1;
            const uint32_t nacc = rb_call(a, slot, myrank, sh, stat, j);
            if (nacc == kNone) {
                suspend = true;
                break;
            }
            done = j;
            if (tid == 0 && a.ccall) a.ccall[slot] = j;
            if (nacc == 0) break;  // no growth: the Hill radius of the unchanged mass stays
            if (!rb_sort_particles(a, slot, sh, stat)) suspend = true;
            else if (a.ck.n && ck_after(j)) rb_checkpoint(a, slot, myrank, j, sh);
        }
        if (!suspend && a.distsq[slot]) {  // the distances of the last sort
            const uint32_t o = a.ct.moff[slot], m = a.ct.mn[slot];
            for (uint32_t k = tid; k < m; k += kRB) a.P.dist[o + k] = sqrt(a.P.dist[o + k]);
            __syncthreads();
            if (tid == 0) a.distsq[slot] = 0;
        }
        __syncthreads();
        if (tid == 0) {
            a.suspended[slot] = suspend ? 1 : 0;
            __threadfence();
            *(volatile uint8_t *)&a.finished[slot] = 1;
        }
        __syncthreads();
    }
}
