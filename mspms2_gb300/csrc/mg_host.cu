// mg_host.cu - context lifecycle, topology expansion, parameters, orchestration and the
// C ABI of the GB300 nonbonded-force engine (include/mspms2_gb300.h).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "mg_internal.cuh"

// ---------------------------------------------------------------------------------
// errors and device buffers
// ---------------------------------------------------------------------------------
mg_status mg_fail(mg_ctx *c, mg_status code, const std::string &msg) {
    if (c) {
        c->err.code = code;
        c->err.msg = msg;
    }
    return code;
}

mg_status mg_cuda_fail(mg_ctx *c, cudaError_t e, const char *what) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return mg_fail(c, e == cudaErrorMemoryAllocation ? MG_ERR_ALLOC : MG_ERR_CUDA, buf);
}

bool mg_ensure(mg_ctx *c, DevBuf &b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return true;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    size_t want = bytes + bytes / 4;  // headroom so small growth does not reallocate
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
        cudaGetLastError();
        mg_fail(c, MG_ERR_ALLOC, "device allocation of " + std::to_string(want) + " bytes failed");
        return false;
    }
    b.bytes = want;
    return true;
}

void mg_free(DevBuf &b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

static mg_status upload(mg_ctx *c, DevBuf &b, const void *src, size_t bytes) {
    if (!mg_ensure(c, b, bytes)) return MG_ERR_ALLOC;
    if (bytes) MG_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// lifecycle
// ---------------------------------------------------------------------------------
extern "C" void mg_options_default(mg_options *o) {
    if (!o) return;
    o->device = 0;
    o->precision = MG_PREC_MIXED;
    o->skin = 0.0;
    o->deterministic = 1;
}

extern "C" int mg_abi_version(void) { return MG_ABI_VERSION; }

extern "C" const char *mg_last_error(const mg_ctx *c) {
    if (!c) return "null context";
    return c->err.msg.c_str();
}

#ifndef MG_FORK_AFTER_LIST
#define MG_FORK_AFTER_LIST 0  // start the reciprocal-space stream after the list build
#endif
#ifndef MG_MAIN_HIGH
#define MG_MAIN_HIGH 1  // the context's own stream at the highest priority
#endif

static bool own_stream_create(cudaStream_t *out) {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return false;
    return cudaStreamCreateWithPriority(out, cudaStreamNonBlocking, MG_MAIN_HIGH ? greatest : least) == cudaSuccess;
}

extern "C" mg_status mg_create(mg_ctx **out, const mg_options *opt) {
    if (!out) return MG_ERR_INVALID;
    *out = nullptr;
    mg_ctx *c = new mg_ctx();
    if (opt)
        c->opt = *opt;
    else
        mg_options_default(&c->opt);
    memset(&c->stats, 0, sizeof(c->stats));
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= c->opt.device || c->opt.device < 0) {
        cudaGetLastError();
        delete c;
        return MG_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c->opt.device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        cudaGetLastError();
        delete c;
        return MG_ERR_NO_DEVICE;  // the kernels are built for sm_103a only
    }
    c->device = c->opt.device;
    if (cudaSetDevice(c->device) != cudaSuccess ||
        !own_stream_create(&c->own_stream)) {
        cudaGetLastError();
        delete c;
        return MG_ERR_CUDA;
    }
    c->stream = c->own_stream;
    for (int i = 0; i < 10; i++) cudaEventCreate(&c->ev[i]);
    c->have_events = true;
    if (!mg_ensure(c, c->d_flags, 64) || !mg_ensure(c, c->d_eout, sizeof(double) * 64)) {
        delete c;
        return MG_ERR_ALLOC;
    }
    *out = c;
    return MG_OK;
}

extern "C" mg_status mg_destroy(mg_ctx *c) {
    if (!c) return MG_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->kstream) cudaStreamSynchronize(c->kstream);
    mg_traj_destroy(c);
    DevBuf *bufs[] = {&c->d_site_mol, &c->d_site_q, &c->d_site_hsig, &c->d_site_seps, &c->d_site_flags,
                      &c->d_site_interp, &c->d_species, &c->d_intra, &c->d_bonded, &c->d_site_aw,
                      &c->d_x, &c->d_y, &c->d_z, &c->d_fl, &c->d_fs, &c->d_xbuild, &c->d_img,
                      &c->d_col_count, &c->d_col_start, &c->d_col_fill, &c->d_col_cl_start, &c->d_col_bkt,
                      &c->d_col_sorted, &c->d_cl_atom, &c->d_cl_ref, &c->d_cl_refh, &c->d_cl_bb, &c->d_cl_col,
                      &c->d_pair_start, &c->d_pair_count, &c->d_pair_j, &c->d_pair_shift,
                      &c->d_pack_pos, &c->d_pack_lj, &c->d_pack_info, &c->d_pack_xi, &c->d_pack_qp, &c->d_rows, &c->d_row_slot,
                      &c->d_phase, &c->d_spart, &c->d_scoef, &c->d_tasks, &c->d_epart, &c->d_eout,
                      &c->d_flags, &c->d_tasos, &c->d_myinterp, &c->d_tubes, &c->d_solid,
                      &c->d_meta, &c->d_pair_img, &c->d_cl_bbf, &c->d_col_ncl, &c->d_counter,
                      &c->d_md_v, &c->d_md_work, &c->d_md_rmass, &c->d_md_part, &c->d_md_dev, &c->d_md_log,
                      &c->d_adj_class, &c->d_adj, &c->d_adj_g,
                      &c->d_sub_start, &c->d_sub_count, &c->d_sub_j, &c->d_sub_shift, &c->d_sub_img, &c->d_facc,
                      &c->d_md_glog, &c->d_fcoef, &c->d_fpart, &c->d_kfb, &c->d_qf, &c->d_fk, &c->d_erows_k};
    for (DevBuf *b : bufs) mg_free(*b);
    c->tasos_buf.clear();  // shared storage is freed by its last holder
    for (auto &b : c->myinterp_buf) mg_free(b);
    if (c->have_events)
        for (int i = 0; i < 10; i++) cudaEventDestroy(c->ev[i]);
    if (c->kstream) {
        cudaStreamDestroy(c->kstream);
        cudaEventDestroy(c->ev_fork);
        cudaEventDestroy(c->ev_join);
    }
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return MG_OK;
}

extern "C" mg_status mg_set_stream(mg_ctx *c, void *stream) {
    if (!c) return MG_ERR_INVALID;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return MG_OK;
}

extern "C" mg_status mg_set_timing(mg_ctx *c, int enable) {
    if (!c) return MG_ERR_INVALID;
    c->timing = enable != 0;
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// parameters (src/initvars.c:591-599, :421-462)
// ---------------------------------------------------------------------------------
extern "C" void mg_params_derive(mg_params *p, double lx, double ly, double lz) {
    if (!p) return;
    const double pi = 3.141592653589793;
    p->rcutoffsq = p->rcutoff * p->rcutoff;
    p->rcutoffelecsq = p->rcutoffelec * p->rcutoffelec;
    p->rcutonsq = p->rcuton * p->rcuton;
    double d = p->rcutoffsq - p->rcutonsq;
    p->roff2_minus_ron2_cube = d * d * d;
    p->shift1 = p->rcutoff > 0 ? pow((1 / p->rcutoff), 6.0) : 0.0;
    p->shift4 = 4.0 * p->shift1;
    p->wolfvcon1 = p->wolfvcon2 = p->wolfvcon3 = p->wolffcon1 = p->wolffcon2 = 0.0;
    p->bfactor_ewald = p->vfactor_ewald = p->twopi_lx = p->twopi_ly = p->twopi_lz = 0.0;
    p->twopi_over_3v = 0.0;
    double k = p->kappa, rc = p->rcutoffelec;
    if (p->charge_type == MG_ELEC_EWALD) {
        p->bfactor_ewald = 1.0 / (4.0 * k * k);
        p->vfactor_ewald = 2.0 * pi / (lx * ly * lz);
        p->twopi_lx = 2.0 * pi / lx;
        p->twopi_ly = 2.0 * pi / ly;
        p->twopi_lz = 2.0 * pi / lz;
        p->twopi_over_3v = 2.0 * pi / 3.0 / lx / ly / lz;
    } else if (p->charge_type == MG_ELEC_WOLF) {
        p->wolfvcon1 = -erfc(k * rc) / rc;
        p->wolfvcon2 = erfc(k * rc) / (rc * rc) + 2.0 * k * exp(-(k * rc) * (k * rc)) / (sqrt(pi) * rc);
        p->wolfvcon3 = k / sqrt(pi) + erfc(k * rc) / (2.0 * rc);
        p->wolffcon1 = 2.0 * k / sqrt(pi);
        p->wolffcon2 = -p->wolfvcon2;
    }
}

extern "C" mg_status mg_set_params(mg_ctx *c, const mg_params *p) {
    if (!c || !p) return MG_ERR_INVALID;
    cudaSetDevice(c->device);
    if (!(p->rcutoff > 0) || !(p->rcutoffelec >= 0) || p->charge_type < 0 || p->charge_type > 3 ||
        p->sf_type < 0 || p->sf_type > 4)
        return mg_fail(c, MG_ERR_INVALID, "invalid cutoffs or model selectors");
    if (p->charge_type == MG_ELEC_EWALD &&
        (p->kmax[0] < 0 || p->kmax[1] < 0 || p->kmax[2] < 0 || p->kmax[0] > 255 || p->kmax[1] > 255 ||
         p->kmax[2] > 255 || p->ksqmax < 0))
        return mg_fail(c, MG_ERR_INVALID, "kmax must lie in [0, 255]");
    if (p->charge_type == MG_ELEC_EWALD && p->ewald_bc != MG_EWALD_BC_TINFOIL && p->ewald_bc != MG_EWALD_BC_VACUUM)
        return mg_fail(c, MG_ERR_INVALID, "ewald_bc must be 1 (tinfoil) or 2 (vacuum)");
    bool kchange = !c->have_params || memcmp(c->params.kmax, p->kmax, sizeof(p->kmax)) != 0 ||
                   c->params.ksqmax != p->ksqmax || c->params.charge_type != p->charge_type;
    bool listchange = !c->have_params || c->params.rcutoff != p->rcutoff ||
                      c->params.rcutoffelec != p->rcutoffelec || c->params.respa_split != p->respa_split;
    c->params = *p;
    c->have_params = true;
    if (listchange) c->list_valid = false;
    if (kchange && p->charge_type == MG_ELEC_EWALD) {
        mg_status s = mg_ewald_setup(c);
        if (s) return s;
    }
    return MG_OK;
}

extern "C" mg_status mg_set_box(mg_ctx *c, double lx, double ly, double lz) {
    if (!c) return MG_ERR_INVALID;
    if (!(lx > 0 && ly > 0 && lz > 0)) return mg_fail(c, MG_ERR_INVALID, "box lengths must be positive");
    if (lx != c->lx || ly != c->ly || lz != c->lz) c->list_valid = false;
    c->lx = lx;
    c->ly = ly;
    c->lz = lz;
    c->have_box = true;
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// topology: the reference's uniqueness rules (src/initvars.c:13-146) and loop order
// (src/frclong.c:228-982, src/frcshort.c:41-84)
// ---------------------------------------------------------------------------------
static void uniqueness(const mg_species &S, std::vector<char> &dih_u, std::vector<char> &agl_u) {
    dih_u.assign(std::max(S.ndih, 0), 1);
    agl_u.assign(std::max(S.nangle, 0), 1);
    auto same_ends = [](int a0, int a1, int b0, int b1) { return (a0 == b0 && a1 == b1) || (a0 == b1 && a1 == b0); };
    for (int i = 0; i + 1 < S.ndih; i++) {
        if (!dih_u[i]) continue;
        for (int j = i + 1; j < S.ndih; j++)
            if (dih_u[j] && same_ends(S.dih_idx[4 * i], S.dih_idx[4 * i + 3], S.dih_idx[4 * j], S.dih_idx[4 * j + 3]))
                dih_u[j] = 0;
    }
    // a dihedral sharing its end pair with an angle or a bond clears the flag of the
    // dihedral whose index equals that angle/bond index (src/initvars.c:66, :86)
    for (int i = 0; i < S.ndih; i++) {
        if (!dih_u[i]) continue;
        for (int j = 0; j < S.nangle; j++)
            if (same_ends(S.dih_idx[4 * i], S.dih_idx[4 * i + 3], S.angle_idx[3 * j], S.angle_idx[3 * j + 2]) && j < S.ndih)
                dih_u[j] = 0;
    }
    for (int i = 0; i < S.ndih; i++) {
        if (!dih_u[i]) continue;
        for (int j = 0; j < S.nbond; j++)
            if (same_ends(S.dih_idx[4 * i], S.dih_idx[4 * i + 3], S.bond_idx[2 * j], S.bond_idx[2 * j + 1]) && j < S.ndih)
                dih_u[j] = 0;
    }
    for (int i = 0; i + 1 < S.nangle; i++) {
        if (!agl_u[i]) continue;
        for (int j = i + 1; j < S.nangle; j++)
            if (agl_u[j] && same_ends(S.angle_idx[3 * i], S.angle_idx[3 * i + 2], S.angle_idx[3 * j], S.angle_idx[3 * j + 2]))
                agl_u[j] = 0;
    }
    for (int i = 0; i < S.nangle; i++) {
        if (!agl_u[i]) continue;
        for (int j = 0; j < S.nbond; j++)  // (src/initvars.c:134)
            if (same_ends(S.angle_idx[3 * i], S.angle_idx[3 * i + 2], S.bond_idx[2 * j], S.bond_idx[2 * j + 1]) && j < S.nangle)
                agl_u[j] = 0;
    }
}

extern "C" mg_status mg_set_topology(mg_ctx *c, int nspecies, const mg_species *sp) {
    if (!c || nspecies <= 0 || !sp) return MG_ERR_INVALID;
    cudaSetDevice(c->device);
    int natom = 0, nmole = 0;
    for (int s = 0; s < nspecies; s++) {
        const mg_species &S = sp[s];
        if (S.natom <= 0 || S.nmole < 0 || S.natom > 4096)
            return mg_fail(c, MG_ERR_INVALID, "species " + std::to_string(s) + ": invalid natom/nmole");
        auto bad_idx = [&](const int *idx, int n, int per) {
            for (int i = 0; i < n * per; i++)
                if (idx[i] < 0 || idx[i] >= S.natom) return true;
            return false;
        };
        if (bad_idx(S.bond_idx, S.nbond, 2) || bad_idx(S.angle_idx, S.nangle, 3) ||
            bad_idx(S.dih_idx, S.ndih, 4) || bad_idx(S.imp_idx, S.nimp, 4) || bad_idx(S.nbp_idx, S.nnbp, 2))
            return mg_fail(c, MG_ERR_INVALID, "species " + std::to_string(s) + ": bonded index out of range");
        for (int b = 0; b < S.nbond; b++)
            if (S.bond_type[b] < 0 || S.bond_type[b] > 3)
                return mg_fail(c, MG_ERR_INVALID, "unknown bond type (src/bndfrc.c:160-162)");
        for (int b = 0; b < S.nangle; b++)
            if (S.angle_type[b] < 0 || S.angle_type[b] > 2)
                return mg_fail(c, MG_ERR_INVALID, "unknown angle type (src/aglfrc.c:188-190)");
        for (int b = 0; b < S.ndih; b++)
            if (S.dih_type[b] < 0 || S.dih_type[b] > 2)
                return mg_fail(c, MG_ERR_INVALID, "unknown dihedral type (src/dihfrc.c:278-280)");
        for (int b = 0; b < S.nimp; b++)
            if (S.imp_type[b] < 0 || S.imp_type[b] > 1)
                return mg_fail(c, MG_ERR_INVALID, "unknown improper type (src/impfrc.c:184-186)");
        natom += S.natom * S.nmole;
        nmole += S.nmole;
    }
    if (natom <= 0) return mg_fail(c, MG_ERR_INVALID, "empty system");
    c->natom = natom;
    c->nmole = nmole;
    c->nspecies = nspecies;
    c->species.clear();
    c->h_tmpl_eps.clear();
    c->h_tmpl_sig.clear();
    c->h_tmpl_aw.clear();
    c->h_site_mol.assign(natom, 0);
    c->h_site_species.assign(natom, 0);
    c->h_site_rel.assign(natom, 0);
    c->h_site_q.assign(natom, 0.0);
    std::vector<double> hs(natom), se(natom), aw(natom);
    std::vector<int> flags(natom), interp(natom);
    std::vector<IntraPair> intra;
    std::vector<BondedTerm> bonded;
    c->has_nbp = false;
    c->max_mol_atoms = 0;
    int site = 0, mole = 0;
    c->sum_q2 = 0.0;
    for (int s = 0; s < nspecies; s++) {
        const mg_species &S = sp[s];
        SpeciesDev d;
        d.natom = S.natom;
        d.nmole = S.nmole;
        d.first_site = site;
        d.first_mole = mole;
        d.mw = 0.0;
        for (int a = 0; a < S.natom; a++) d.mw += S.aw[a];
        std::vector<char> dih_u, agl_u;
        uniqueness(S, dih_u, agl_u);
        d.intra_off = (int)intra.size();
        for (int b = 0; b < S.nbond; b++) intra.push_back({S.bond_idx[2 * b], S.bond_idx[2 * b + 1], 0});
        for (int g = 0; g < S.nangle; g++)
            if (agl_u[g]) intra.push_back({S.angle_idx[3 * g], S.angle_idx[3 * g + 2], 0});
        for (int q = 0; q < S.ndih; q++)
            if (dih_u[q]) intra.push_back({S.dih_idx[4 * q], S.dih_idx[4 * q + 3], 1});
        for (int q = 0; q < S.nnbp; q++) {
            // nbp pair source (src/frclong.c:793-794 reads entry ndih for every q)
            int src = (c->params.compat & MG_COMPAT_NBP_INDEX) ? S.ndih : q;
            int m = 0, n = 0;
            if (src < S.nnbp) {
                m = S.nbp_idx[2 * src];
                n = S.nbp_idx[2 * src + 1];
            }
            intra.push_back({m, n, 2});
            c->has_nbp = true;
        }
        d.nintra = (int)intra.size() - d.intra_off;
        d.bonded_off = (int)bonded.size();
        for (int b = 0; b < S.nbond; b++) {
            BondedTerm t{};
            t.kind = 0;
            t.type = S.bond_type[b];
            t.idx[0] = S.bond_idx[2 * b];
            t.idx[1] = S.bond_idx[2 * b + 1];
            for (int k = 0; k < 3; k++) t.p[k] = S.bond_param[3 * b + k];
            bonded.push_back(t);
        }
        for (int g = 0; g < S.nangle; g++) {
            BondedTerm t{};
            t.kind = 1;
            t.type = S.angle_type[g];
            for (int k = 0; k < 3; k++) t.idx[k] = S.angle_idx[3 * g + k];
            for (int k = 0; k < 5; k++) t.p[k] = S.angle_param[5 * g + k];
            bonded.push_back(t);
        }
        for (int q = 0; q < S.ndih; q++) {
            BondedTerm t{};
            t.kind = 2;
            t.type = S.dih_type[q];
            for (int k = 0; k < 4; k++) t.idx[k] = S.dih_idx[4 * q + k];
            for (int k = 0; k < 4; k++) t.p[k] = S.dih_param[4 * q + k];
            bonded.push_back(t);
        }
        for (int q = 0; q < S.nimp; q++) {
            BondedTerm t{};
            t.kind = 3;
            t.type = S.imp_type[q];
            for (int k = 0; k < 4; k++) t.idx[k] = S.imp_idx[4 * q + k];
            for (int k = 0; k < 2; k++) t.p[k] = S.imp_param[2 * q + k];
            bonded.push_back(t);
        }
        d.nbonded = (int)bonded.size() - d.bonded_off;
        c->max_mol_atoms = std::max(c->max_mol_atoms, S.natom);
        c->h_tmpl_eps.emplace_back(S.epsilon, S.epsilon + S.natom);
        c->h_tmpl_sig.emplace_back(S.sigma, S.sigma + S.natom);
        c->h_tmpl_aw.emplace_back();
        for (int a = 0; a < S.natom; a++) c->h_tmpl_aw.back().push_back(S.aw ? S.aw[a] : 1.0);
        for (int m = 0; m < S.nmole; m++, mole++)
            for (int a = 0; a < S.natom; a++, site++) {
                c->h_site_mol[site] = mole;
                c->h_site_species[site] = s;
                c->h_site_rel[site] = a;
                c->h_site_q[site] = S.charge[a];
                c->sum_q2 += S.charge[a] * S.charge[a];
                hs[site] = 0.5 * S.sigma[a];
                se[site] = sqrt(S.epsilon[a]);
                int g = S.ghost_type[a];
                flags[site] = (g == MG_GHOST_FULL ? MG_SITE_DEAD : 0) |
                              ((g != MG_GHOST_LJ && g != MG_GHOST_FULL) ? MG_SITE_LJ : 0) |
                              (g == MG_GHOST_NONE ? 4 : 0);  // bit 2: solid-fluid active
                interp[site] = S.interp_type ? S.interp_type[a] : 0;
                aw[site] = S.aw ? S.aw[a] : 1.0;
            }
        c->species.push_back(d);
    }
    mg_status st;
    if ((st = upload(c, c->d_site_mol, c->h_site_mol.data(), sizeof(int) * natom))) return st;
    if ((st = upload(c, c->d_site_q, c->h_site_q.data(), sizeof(double) * natom))) return st;
    if ((st = upload(c, c->d_site_hsig, hs.data(), sizeof(double) * natom))) return st;
    if ((st = upload(c, c->d_site_seps, se.data(), sizeof(double) * natom))) return st;
    if ((st = upload(c, c->d_site_flags, flags.data(), sizeof(int) * natom))) return st;
    if ((st = upload(c, c->d_site_interp, interp.data(), sizeof(int) * natom))) return st;
    if ((st = upload(c, c->d_site_aw, aw.data(), sizeof(double) * natom))) return st;
    if ((st = upload(c, c->d_species, c->species.data(), sizeof(SpeciesDev) * c->species.size()))) return st;
    if ((st = upload(c, c->d_intra, intra.data(), sizeof(IntraPair) * intra.size()))) return st;
    if ((st = upload(c, c->d_bonded, bonded.data(), sizeof(BondedTerm) * bonded.size()))) return st;
    c->have_topology = true;
    c->list_valid = false;
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// solid-fluid tables
// ---------------------------------------------------------------------------------
extern "C" mg_status mg_sf_tasos_set_grid(mg_ctx *c, int type, int nx, int ny, int nz, double hx,
                                          double hy, double hz, double cuc, const double *values) {
    if (!c || type < 1 || type > 64 || nx < 3 || ny < 3 || nz < 3 || !(hx > 0) || !(hy > 0) || !(hz > 0) ||
        !(cuc > 0) || !values)
        return mg_fail(c, MG_ERR_INVALID, "invalid Tasos grid");
    cudaSetDevice(c->device);
    if ((int)c->tasos.size() < type) {
        c->tasos.resize(type);
        c->tasos_buf.resize(type);
    }
    size_t nn = (size_t)nx * ny * nz;
    double mn = 10e10;  // minPE of mylibtasos/grid.f90:75-97
    for (size_t i = 0; i < nn; i++) mn = std::min(mn, values[8 * i]);
    TasosDev &t = c->tasos[type - 1];
    t.nx = nx; t.ny = ny; t.nz = nz;
    t.hx = hx; t.hy = hy; t.hz = hz; t.cuc = cuc; t.min_pe = mn;
    mg_status st;
    DevBuf &buf = mg_tasos_storage(c, type);
    if (c->opt.precision == MG_PREC_FP64) {
        if ((st = upload(c, buf, values, sizeof(double) * 8 * nn))) return st;
    } else {
        std::vector<float> f(8 * nn);
        for (size_t i = 0; i < 8 * nn; i++) f[i] = (float)values[i];
        if ((st = upload(c, buf, f.data(), sizeof(float) * 8 * nn))) return st;
    }
    t.values = buf.p;
    return upload(c, c->d_tasos, c->tasos.data(), sizeof(TasosDev) * c->tasos.size());
}

DevBuf &mg_tasos_storage(mg_ctx *c, int type) {
    std::shared_ptr<DevBuf> &p = c->tasos_buf[type - 1];
    if (!p || p.use_count() > 1)
        p = std::shared_ptr<DevBuf>(new DevBuf(), [](DevBuf *b) {
            mg_free(*b);
            delete b;
        });
    return *p;
}

extern "C" mg_status mg_sf_tasos_share(mg_ctx *dst, const mg_ctx *src) {
    if (!dst || !src || dst == src) return MG_ERR_INVALID;
    if (dst->device != src->device || dst->opt.precision != src->opt.precision)
        return mg_fail(dst, MG_ERR_INVALID, "Tasos tables can be shared only between contexts of one device and precision");
    cudaSetDevice(dst->device);
    dst->tasos = src->tasos;
    dst->tasos_buf = src->tasos_buf;
    if (dst->tasos.empty()) return MG_OK;
    return upload(dst, dst->d_tasos, dst->tasos.data(), sizeof(TasosDev) * dst->tasos.size());
}

extern "C" mg_status mg_sf_hypergeo_set(mg_ctx *c, int ntube, const double *cx, const double *cy,
                                        const double *radius, double solid_sigma, double solid_epsilon,
                                        double const_3pisq_theta) {
    if (!c || ntube < 0 || (ntube > 0 && (!cx || !cy || !radius))) return MG_ERR_INVALID;
    cudaSetDevice(c->device);
    std::vector<double> t(3 * (size_t)std::max(ntube, 1));
    for (int i = 0; i < ntube; i++) {
        t[3 * i] = cx[i];
        t[3 * i + 1] = cy[i];
        t[3 * i + 2] = radius[i];
    }
    c->ntube = ntube;
    c->solid_sigma = solid_sigma;
    c->solid_epsilon = solid_epsilon;
    c->const_3pisq_theta = const_3pisq_theta;
    return upload(c, c->d_tubes, t.data(), sizeof(double) * t.size());
}

extern "C" mg_status mg_sf_atom_explicit_set(mg_ctx *c, int nsolid, const double *sx, const double *sy,
                                             const double *sz, double solid_sigma, double solid_epsilon) {
    if (!c || nsolid < 0 || (nsolid > 0 && (!sx || !sy || !sz))) return MG_ERR_INVALID;
    cudaSetDevice(c->device);
    std::vector<double> t(3 * (size_t)std::max(nsolid, 1));
    for (int i = 0; i < nsolid; i++) {
        t[3 * i] = sx[i];
        t[3 * i + 1] = sy[i];
        t[3 * i + 2] = sz[i];
    }
    c->nsolid = nsolid;
    c->solid_sigma = solid_sigma;
    c->solid_epsilon = solid_epsilon;
    return upload(c, c->d_solid, t.data(), sizeof(double) * t.size());
}

extern "C" mg_status mg_sf_myinterp_set(mg_ctx *c, int type, int ncx, int ncy, int ncz, double itvl_x,
                                        double itvl_y, double itvl_z, double xmin, double ymin, double zmax,
                                        const double *coeff) {
    if (!c || type < 0 || type > 63 || ncx <= 0 || ncy <= 0 || ncz <= 0 || !coeff)
        return mg_fail(c, MG_ERR_INVALID, "invalid my-interp grid");
    cudaSetDevice(c->device);
    if ((int)c->myinterp.size() <= type) {
        c->myinterp.resize(type + 1);
        c->myinterp_buf.resize(type + 1);
    }
    size_t ncube = (size_t)ncx * ncy * ncz;
    mg_status st;
    if ((st = upload(c, c->myinterp_buf[type], coeff, sizeof(double) * 128 * ncube))) return st;
    MyInterpDev &m = c->myinterp[type];
    m.ncx = ncx; m.ncy = ncy; m.ncz = ncz;
    m.itvl_x = itvl_x; m.itvl_y = itvl_y; m.itvl_z = itvl_z;
    m.xmin = xmin; m.ymin = ymin; m.zmax = zmax;
    m.coeff = (double *)c->myinterp_buf[type].p;
    return upload(c, c->d_myinterp, c->myinterp.data(), sizeof(MyInterpDev) * c->myinterp.size());
}

// ---------------------------------------------------------------------------------
// evaluation
// ---------------------------------------------------------------------------------
static void assemble_energies(mg_ctx *c, const double *E, int want_long, int want_short, mg_energies *e) {
    const mg_params &p = c->params;
    const double pi = 3.141592653589793;
    memset(e, 0, sizeof(*e));
    bool split = p.respa_split > 0;
    if (want_long) {
        e->uvdw = E[E_UVDW];
        e->ushift = E[E_USHIFT];
        e->ureal = E[E_UREAL];
        e->uexcl = E[E_UEXCL];
        e->virial_inter = E[E_VIR];
        if (p.charge_type == MG_ELEC_EWALD) {
            e->ufourier = E[E_UFOURIER];
            e->uself = c->sum_q2 * (p.coulomb_prefactor * sqrt(p.kappa * p.kappa / pi));
            e->uelec = e->ureal + e->ufourier - e->uself - e->uexcl;
            if (p.ewald_bc == MG_EWALD_BC_VACUUM) {
                double mx = E[E_DIPX], my = E[E_DIPY], mz = E[E_DIPZ];
                e->uvacuum = (mx * mx + my * my + mz * mz) * p.twopi_over_3v * p.coulomb_prefactor;
                e->uelec += e->uvacuum;
            }
        } else if (p.charge_type == MG_ELEC_WOLF) {
            e->uself = c->sum_q2 * (p.coulomb_prefactor * p.wolfvcon3);
            e->uelec = e->ureal - e->uself - e->uexcl;
        } else if (p.charge_type == MG_ELEC_SIMPLE_COULOMB) {
            e->uelec = E[E_UCOUL];
        }
        e->usflj = E[E_USFLJ];
    }
    if (split && want_short) {
        e->uvdw += E[E_UVDW_S];
        e->ushift += E[E_USHIFT_S];
        e->ureal += E[E_UREAL_S];
        e->virial_inter += E[E_VIR_S];
        if (p.charge_type == MG_ELEC_EWALD || p.charge_type == MG_ELEC_WOLF) e->uelec += E[E_UREAL_S];
    }
    e->ushift *= p.shift4;
    if (p.charge_type == MG_ELEC_EWALD && (want_long || split)) {
        // the reference adds the whole Ewald energy as the electrostatic virial
        // (src/frclong.c:1128); the short bucket carries its real-space share
        double eshort = (split && want_short) ? E[E_UREAL_S] : 0.0;
        double elong = want_long ? e->uelec - eshort : 0.0;
        e->virial_inter += elong + eshort;
    }
    e->uotherff = 0.0;
    e->uinter = e->uvdw + e->uelec + e->usflj + e->uotherff;
    if (want_short) {
        e->ubond = E[E_UBOND];
        e->uangle = E[E_UANGLE];
        e->udih = E[E_UDIH];
        e->uimp = E[E_UIMP];
        e->virial_intra = E[E_VIR_INTRA];
        e->uintra = e->ubond + e->uangle + e->udih + e->uimp;
    }
}

// One attempt; *retry is set when the list set-up must change and the call be repeated.
void mg_assemble_energies(mg_ctx *c, const double *E, int want_long, int want_short, mg_energies *e) {
    assemble_energies(c, E, want_long, want_short, e);
}

// Every launch of one evaluation, in order, on the context's stream, with no host
// synchronisation (so that it can also be captured into a graph): the raw energy
// components end in d_eout, the error flags in d_flags, the list counts in d_meta.
mg_status mg_enqueue_forces(mg_ctx *c, const double *dx, const double *dy, const double *dz, int terms, double *fl,
                            double *fs) {
    if (!c->have_topology || !c->have_params || !c->have_box)
        return mg_fail(c, MG_ERR_STATE, "set topology, params and box before computing");
    const mg_params &p = c->params;
    if (p.charge_type == MG_ELEC_EWALD && (c->lx != c->ewald_box[0] || c->ly != c->ewald_box[1] || c->lz != c->ewald_box[2])) {
        mg_status s = mg_ewald_setup(c);
        if (s) return s;
    }
    int want_long = (terms & MG_TERMS_LONG) != 0;
    int want_short = (terms & MG_TERMS_SHORT) != 0;
    bool split = p.respa_split > 0;
    if (p.sf_type == MG_SF_TASOS && c->tasos.empty()) return mg_fail(c, MG_ERR_STATE, "Tasos grids not loaded");
    if (p.sf_type == MG_SF_MY_INTERP && c->myinterp.empty()) return mg_fail(c, MG_ERR_STATE, "my-interp grids not loaded");
    cudaStream_t s = c->stream;
    MG_CUDA(cudaMemsetAsync(c->d_flags.p, 0, 64, s));
    if (c->timing) cudaEventRecord(c->ev[0], s);
    c->list_rebuilt = 0;
    c->launches = 0;
    bool need_pairs = want_long || (split && want_short);
    mg_status st;
    const bool ewald = want_long && p.charge_type == MG_ELEC_EWALD;
    c->forked = false;
    const bool fork = ewald && c->kspace_overlap && c->nrows > 0;
    if (fork && !MG_FORK_AFTER_LIST && (st = mg_ewald_fork(c, dx, dy, dz))) return st;
    if (need_pairs) {
        if ((st = mg_list_update(c, dx, dy, dz))) return st;
        if ((st = mg_pack_clusters(c, dx, dy, dz))) return st;
    }
    // energy partial rows: an upper bound of the blocks every stage may launch
    {
        long long rows = (need_pairs ? (c->cl_cap + 3) / 4 : 0) + 4LL * ((c->nmole + 127) / 128) +
                         (c->natom + 127) / 128 + (c->nslots + 255) / 256 + 16;
        if (!mg_ensure(c, c->d_epart, sizeof(double) * E_NCOMP * (size_t)rows)) return MG_ERR_ALLOC;
        c->epart_cap = (int)(c->d_epart.bytes / (sizeof(double) * E_NCOMP));
        c->epart_rows = 0;
    }
    if (c->timing) cudaEventRecord(c->ev[1], s);
    if (fork && MG_FORK_AFTER_LIST && (st = mg_ewald_fork(c, dx, dy, dz))) return st;
    if (need_pairs) {
        if ((st = mg_launch_pair(c, want_long, split && want_short, want_long ? fl : nullptr,
                                 (split && want_short) ? fs : nullptr)))
            return st;
    }
    if (c->timing) cudaEventRecord(c->ev[2], s);
    if (want_short && !split) MG_CUDA(cudaMemsetAsync(fs, 0, sizeof(double) * 3 * c->natom, s));
    if (want_long) {
        if ((st = mg_launch_intra(c, dx, dy, dz, fl))) return st;
        if (p.charge_type == MG_ELEC_SIMPLE_COULOMB && (st = mg_launch_coulomb_mole(c, dx, dy, dz, fl))) return st;
    }
    if (want_short && (st = mg_launch_bonded(c, dx, dy, dz, fs))) return st;
    if (c->timing) cudaEventRecord(c->forked ? c->ev[8] : c->ev[3], s);
    if (ewald) {
        if (c->forked) {
            if ((st = mg_ewald_join(c, fl))) return st;
        } else if ((st = mg_launch_ewald(c, dx, dy, dz, fl))) {  // records ev[4] after the S(k) reduction
            return st;
        }
        if (p.ewald_bc == MG_EWALD_BC_VACUUM && (st = mg_launch_vacuum(c, dx, dy, dz, fl))) return st;
    } else if (c->timing) {
        cudaEventRecord(c->ev[4], s);
    }
    if (c->timing) cudaEventRecord(c->forked ? c->ev[9] : c->ev[5], s);
    if (want_long && p.sf_type != MG_SF_NONE && (st = mg_launch_sf(c, dx, dy, dz, fl))) return st;
    if (c->timing) cudaEventRecord(c->ev[6], s);
    if ((st = mg_launch_reduce(c))) return st;
    if (want_long && (st = mg_launch_check(c, fl, c->natom))) return st;
    if (want_short && (st = mg_launch_check(c, fs, c->natom))) return st;
    if (c->timing) cudaEventRecord(c->ev[7], s);
    return MG_OK;
}

static mg_status compute_once(mg_ctx *c, const double *dx, const double *dy, const double *dz, int terms,
                              double *fl, double *fs, mg_energies *e, bool *retry) {
    *retry = false;
    mg_status st = mg_enqueue_forces(c, dx, dy, dz, terms, fl, fs);
    if (st) return st;
    const mg_params &p = c->params;
    cudaStream_t s = c->stream;
    int want_long = (terms & MG_TERMS_LONG) != 0;
    int want_short = (terms & MG_TERMS_SHORT) != 0;
    bool split = p.respa_split > 0;
    bool need_pairs = want_long || (split && want_short);
    double E[E_NCOMP + 8];
    unsigned flags[4];
    int meta[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    MG_CUDA(cudaMemcpyAsync(E, c->d_eout.p, sizeof(double) * E_NCOMP, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(flags, c->d_flags.p, sizeof(unsigned) * 4, cudaMemcpyDeviceToHost, s));
    if (need_pairs) MG_CUDA(cudaMemcpyAsync(meta, c->d_meta.p, sizeof(meta), cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    MG_CUDA(cudaGetLastError());
    c->last_flags = flags[0];
    if (need_pairs) {
        if (mg_list_retry(c, flags[0], meta)) {
            *retry = true;
            return MG_OK;
        }
        if (flags[0] & MG_FLAG_FIXED_RANGE) {
            // a pair force outside the range of the fixed-point force sums: a coarser unit
            // (2^-32, then 2^-16, then 1), kept by the context for later calls, and the call again
            if (c->fixed_bits <= 0)
                return mg_fail(c, MG_ERR_NONFINITE, "pair force beyond the range of the fixed-point force sums");
            c->fixed_bits -= 16;
            *retry = true;
            return MG_OK;
        }
        c->ncl = meta[0];
        c->npairs = c->small_box ? (long long)meta[0] * meta[0] : *(long long *)(meta + 4);
        c->list_rebuilt = meta[3] != c->list_builds;
        c->list_builds = meta[3];
    }
    mg_energies en;
    assemble_energies(c, E, want_long, want_short, &en);
    if (e) *e = en;
    c->stats.pairs_within_cutoff = need_pairs ? (long long)(E[E_NPAIR] * 0.5 + 0.25) : 0;
    c->stats.list_rebuilt = c->list_rebuilt;
    c->stats.list_builds = c->list_builds;
    c->stats.nclusters = c->ncl;
    c->stats.cluster_pairs = c->npairs;
    c->stats.kvectors = p.charge_type == MG_ELEC_EWALD ? c->kvectors : 0;
    c->stats.kernel_launches = c->launches;
    if (c->timing) {
        float ms;
        for (int i = 0; i < 7; i++) {
            cudaEventElapsedTime(&ms, c->ev[i], c->ev[i + 1]);
            c->stats.kernel_ms[i] = ms;
        }
        if (c->forked) {  // S(k) and k-forces on their own stream (ev 3-5), beside pairs
            cudaEventElapsedTime(&ms, c->ev[2], c->ev[8]);
            c->stats.kernel_ms[2] = ms;
            cudaEventElapsedTime(&ms, c->ev[9], c->ev[6]);
            c->stats.kernel_ms[5] = ms;
        }
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[7]);
        c->stats.kernel_ms[7] = ms;
    }
    if (flags[0] & MG_FLAG_OUT_OF_GRID)
        return mg_fail(c, MG_ERR_OUT_OF_GRID, "a site left its solid-fluid table");
    if (flags[0] & MG_FLAG_IMPROPER_DEGENERATE)
        return mg_fail(c, MG_ERR_INVALID, "degenerate CHARMM improper (src/impfrc.c:96-134 exits here)");
    if (flags[0] & (MG_FLAG_LIST_OVERFLOW | MG_FLAG_COLUMN_OVERFLOW))
        return mg_fail(c, MG_ERR_CAPACITY, "neighbour-list capacity exceeded");
    // a give-up of a tensor-core reciprocal-space pass (S(k) or forces) spoils the forces: report the cause
    if (flags[0] & MG_FLAG_MMA_UNDRAINED)
        return mg_fail(c, MG_ERR_CUDA, "tensor-core reciprocal-space pass: an on-chip wait ran out and issued MMAs did "
                                       "not finish within the bound (tensor memory of the launch may have been overwritten)");
    if (flags[0] & MG_FLAG_WAIT_TIMEOUT)
        return mg_fail(c, MG_ERR_CUDA, "tensor-core reciprocal-space pass: an on-chip wait ran out");
    if (flags[0] & MG_FLAG_NONFINITE) return mg_fail(c, MG_ERR_NONFINITE, "non-finite force");
    return MG_OK;
}

mg_status mg_compute_forces(mg_ctx *c, const double *dx, const double *dy, const double *dz, int terms,
                              double *fl, double *fs, mg_energies *e) {
    for (int attempt = 0; attempt < 6; attempt++) {
        bool retry = false;
        mg_status st = compute_once(c, dx, dy, dz, terms, fl, fs, e, &retry);
        if (st || !retry) return st;
    }
    return mg_fail(c, MG_ERR_CAPACITY, "neighbour-list set-up did not converge");
}

extern "C" mg_status mg_compute_device(mg_ctx *c, const double *dx, const double *dy, const double *dz,
                                       int terms, double *fxl, double *fyl, double *fzl, double *fxs,
                                       double *fys, double *fzs, mg_energies *e) {
    if (!c || !dx || !dy || !dz || !(terms & MG_TERMS_ALL)) return MG_ERR_INVALID;
    cudaSetDevice(c->device);
    // the kernels use [3][n] force blocks; device callers may pass any three pointers,
    // so results go through the context's blocks and are copied out
    size_t nb = sizeof(double) * c->natom;
    if (!mg_ensure(c, c->d_fl, 3 * nb) || !mg_ensure(c, c->d_fs, 3 * nb)) return MG_ERR_ALLOC;
    double *fl = (double *)c->d_fl.p, *fs = (double *)c->d_fs.p;
    mg_status st = mg_compute_forces(c, dx, dy, dz, terms, fl, fs, e);
    if (st && st != MG_ERR_NONFINITE) return st;
    cudaStream_t s = c->stream;
    if ((terms & MG_TERMS_LONG) && fxl && fyl && fzl) {
        if (fxl != fl) MG_CUDA(cudaMemcpyAsync(fxl, fl, nb, cudaMemcpyDeviceToDevice, s));
        if (fyl != fl + c->natom) MG_CUDA(cudaMemcpyAsync(fyl, fl + c->natom, nb, cudaMemcpyDeviceToDevice, s));
        if (fzl != fl + 2 * c->natom) MG_CUDA(cudaMemcpyAsync(fzl, fl + 2 * c->natom, nb, cudaMemcpyDeviceToDevice, s));
    }
    if ((terms & MG_TERMS_SHORT) && fxs && fys && fzs) {
        if (fxs != fs) MG_CUDA(cudaMemcpyAsync(fxs, fs, nb, cudaMemcpyDeviceToDevice, s));
        if (fys != fs + c->natom) MG_CUDA(cudaMemcpyAsync(fys, fs + c->natom, nb, cudaMemcpyDeviceToDevice, s));
        if (fzs != fs + 2 * c->natom) MG_CUDA(cudaMemcpyAsync(fzs, fs + 2 * c->natom, nb, cudaMemcpyDeviceToDevice, s));
    }
    return st;
}

extern "C" mg_status mg_compute(mg_ctx *c, const double *x, const double *y, const double *z, int terms,
                                double *fxl, double *fyl, double *fzl, double *fxs, double *fys, double *fzs,
                                mg_energies *e) {
    if (!c || !x || !y || !z || !(terms & MG_TERMS_ALL)) return MG_ERR_INVALID;
    if ((terms & MG_TERMS_LONG) && !(fxl && fyl && fzl)) return mg_fail(c, MG_ERR_INVALID, "long force arrays missing");
    if ((terms & MG_TERMS_SHORT) && !(fxs && fys && fzs)) return mg_fail(c, MG_ERR_INVALID, "short force arrays missing");
    if (!c->have_topology) return mg_fail(c, MG_ERR_STATE, "no topology");
    cudaSetDevice(c->device);
    size_t nb = sizeof(double) * c->natom;
    if (!mg_ensure(c, c->d_x, 3 * nb) || !mg_ensure(c, c->d_fl, 3 * nb) || !mg_ensure(c, c->d_fs, 3 * nb))
        return MG_ERR_ALLOC;
    double *dx = (double *)c->d_x.p, *dy = dx + c->natom, *dz = dy + c->natom;
    cudaStream_t s = c->stream;
    MG_CUDA(cudaMemcpyAsync(dx, x, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(dy, y, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(dz, z, nb, cudaMemcpyHostToDevice, s));
    double *fl = (double *)c->d_fl.p, *fs = (double *)c->d_fs.p;
    mg_status st = mg_compute_forces(c, dx, dy, dz, terms, fl, fs, e);
    if (st && st != MG_ERR_NONFINITE) return st;
    if (terms & MG_TERMS_LONG) {
        MG_CUDA(cudaMemcpyAsync(fxl, fl, nb, cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaMemcpyAsync(fyl, fl + c->natom, nb, cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaMemcpyAsync(fzl, fl + 2 * c->natom, nb, cudaMemcpyDeviceToHost, s));
    }
    if (terms & MG_TERMS_SHORT) {
        MG_CUDA(cudaMemcpyAsync(fxs, fs, nb, cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaMemcpyAsync(fys, fs + c->natom, nb, cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaMemcpyAsync(fzs, fs + 2 * c->natom, nb, cudaMemcpyDeviceToHost, s));
    }
    MG_CUDA(cudaStreamSynchronize(s));
    return st;
}

extern "C" mg_status mg_get_stats(const mg_ctx *c, mg_stats *s) {
    if (!c || !s) return MG_ERR_INVALID;
    *s = c->stats;
    return MG_OK;
}

extern "C" mg_status mg_get_device_flags(const mg_ctx *c, unsigned *flags) {
    if (!c || !flags) return MG_ERR_INVALID;
    *flags = c->last_flags;
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// autotuning of the launch geometry
// ---------------------------------------------------------------------------------
static void tuning_out(const mg_ctx *c, mg_tuning *t) {
    t->cell_scale = c->tune.cell_scale;
    t->zcap_scale = c->tune.zcap_scale;
    t->kforce_threads = c->tune.kforce_threads;
}

extern "C" mg_status mg_get_tuning(const mg_ctx *c, mg_tuning *t) {
    if (!c || !t) return MG_ERR_INVALID;
    memset(t, 0, sizeof(*t));
    tuning_out(c, t);
    return MG_OK;
}

extern "C" mg_status mg_set_tuning(mg_ctx *c, const mg_tuning *t) {
    if (!c || !t) return MG_ERR_INVALID;
    if (!(t->cell_scale >= 0.5 && t->cell_scale <= 2.0) || !(t->zcap_scale >= 0.5 && t->zcap_scale <= 2.0) ||
        !(t->kforce_threads == 2 || t->kforce_threads == 4 || t->kforce_threads == 8))
        return mg_fail(c, MG_ERR_INVALID, "tuning out of range (scales 0.5-2, threads 2, 4 or 8)");
    c->tune.cell_scale = t->cell_scale;
    c->tune.zcap_scale = t->zcap_scale;
    c->tune.kforce_threads = t->kforce_threads;
    c->tune.tuned = true;
    c->list_valid = false;  // the grid follows the new geometry at the next call
    return MG_OK;
}

extern "C" mg_status mg_autotune(mg_ctx *c, const double *x, const double *y, const double *z, int terms,
                                 mg_tuning *out) {
    if (!c || !x || !y || !z || !(terms & MG_TERMS_ALL)) return MG_ERR_INVALID;
    if (!c->have_topology || !c->have_params || !c->have_box)
        return mg_fail(c, MG_ERR_STATE, "set topology, params and box before tuning");
    cudaSetDevice(c->device);
    const size_t nb = sizeof(double) * c->natom;
    if (!mg_ensure(c, c->d_x, 3 * nb) || !mg_ensure(c, c->d_fl, 3 * nb) || !mg_ensure(c, c->d_fs, 3 * nb))
        return MG_ERR_ALLOC;
    double *dx = (double *)c->d_x.p, *dy = dx + c->natom, *dz = dy + c->natom;
    cudaStream_t s = c->stream;
    MG_CUDA(cudaMemcpyAsync(dx, x, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(dy, y, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(dz, z, nb, cudaMemcpyHostToDevice, s));
    cudaEvent_t e0, e1;
    MG_CUDA(cudaEventCreate(&e0));
    MG_CUDA(cudaEventCreate(&e1));
    int tried = 0;
    // one evaluation (after one untimed call that rebuilds the list for the geometry):
    // the fastest of three, so that one slow launch does not decide
    auto timed = [&](float *ms) -> mg_status {
        c->list_valid = false;
        mg_status st = mg_compute_forces(c, dx, dy, dz, terms, (double *)c->d_fl.p, (double *)c->d_fs.p, nullptr);
        if (st) return st;
        float best = 1e30f;
        for (int r = 0; r < 3; r++) {
            MG_CUDA(cudaEventRecord(e0, s));
            if ((st = mg_compute_forces(c, dx, dy, dz, terms, (double *)c->d_fl.p, (double *)c->d_fs.p, nullptr)))
                return st;
            MG_CUDA(cudaEventRecord(e1, s));
            MG_CUDA(cudaEventSynchronize(e1));
            float t = 0.f;
            MG_CUDA(cudaEventElapsedTime(&t, e0, e1));
            best = std::min(best, t);
        }
        tried++;
        *ms = best;
        return MG_OK;
    };
    const MgTuning keep = c->tune;
    c->tune = MgTuning();
    float base = 0.f, ms = 0.f;
    mg_status st = timed(&base);
    MgTuning best = c->tune;
    float best_ms = base;
    // threads per site matter only to the Horner k-force pass (FP64, or rows too long for
    // the FP32 table pass)
    if (!st && c->params.charge_type == MG_ELEC_EWALD && (terms & MG_TERMS_LONG) && mg_ewald_horner_force(c)) {
        for (int fg : {2, 8}) {
            c->tune = best;
            c->tune.kforce_threads = fg;
            if ((st = timed(&ms))) break;
            if (ms < best_ms) {
                best_ms = ms;
                best = c->tune;
            }
        }
    }
    const double cells[3] = {0.8, 1.0, 1.25}, zcaps[3] = {0.75, 1.0, 1.5};
    const MgTuning row = best;
    for (int i = 0; i < 3 && !st; i++)
        for (int j = 0; j < 3 && !st; j++) {
            if (cells[i] == 1.0 && zcaps[j] == 1.0) continue;  // measured above
            c->tune = row;
            c->tune.cell_scale = cells[i];
            c->tune.zcap_scale = zcaps[j];
            if ((st = timed(&ms))) break;
            if (ms < best_ms) {
                best_ms = ms;
                best = c->tune;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) {
        c->tune = keep;
        c->list_valid = false;
        return st;
    }
    c->tune = best;
    c->tune.tuned = true;
    c->list_valid = false;
    if (out) {
        tuning_out(c, out);
        out->ms_default = base;
        out->ms_tuned = best_ms;
        out->configs_tried = tried;
    }
    return MG_OK;
}

extern "C" mg_status mg_set_kspace_overlap(mg_ctx *c, int enable) {
    if (!c) return MG_ERR_INVALID;
    c->kspace_overlap = enable != 0;
    return MG_OK;
}

extern "C" mg_status mg_set_kspace_tensor(mg_ctx *c, int enable) {
    if (!c) return MG_ERR_INVALID;
    c->kspace_tensor = enable != 0;
    return MG_OK;
}

// polls of each on-chip pipeline wait of the tensor-core S(k) pass, process-wide; read at
// every launch (the default bounds a wait to well under a second)
static std::atomic<long long> g_wait_limit{1ll << 20};

long long mg_wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }

extern "C" mg_status mg_set_wait_limit(long long polls) {
    g_wait_limit.store(polls < 0 ? (1ll << 20) : polls, std::memory_order_relaxed);
    return MG_OK;
}

extern "C" mg_status mg_set_md_graphs(mg_ctx *c, int enable) {
    if (!c) return MG_ERR_INVALID;
    c->md_graphs = enable != 0;
    return MG_OK;
}

extern "C" mg_status mg_get_md_graphs(const mg_ctx *c, int *enabled, int *last_steps) {
    if (!c) return MG_ERR_INVALID;
    if (enabled) *enabled = c->md_graphs ? 1 : 0;
    if (last_steps) *last_steps = c->md_graph_steps;
    return MG_OK;
}
