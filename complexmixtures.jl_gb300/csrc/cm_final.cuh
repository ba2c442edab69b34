// cm_final.cuh -- finalisation of accumulated counts on the device (FP64).
//
// Restates finalresults! (src/results.jl:311-318): _mddf_final_results!
// (src/results.jl:320-376) with renormalize! (src/results.jl:378-428), and
// _coordination_number_final_results! (src/results.jl:430-469).  One CTA per
// job, so many requests are finalised in one launch.  Elementwise steps run
// over the threads; every sum and cumulative sum runs on one thread in index
// order, as the reference's loops do, so the results equal the host's
// sequential FP64 arithmetic (the shell radius takes the device's pow).
#pragma once
#include "cm_kernels.cuh"

namespace cmk {

// Offsets of the packed output of a job ([nbins] blocks, then the group
// blocks, then the scalars).
enum FinalVec {
    FV_D = 0, FV_MD, FV_MDR, FV_CN, FV_CNR, FV_MDDF, FV_KB, FV_RDFC, FV_RDFCR, FV_SRDF, FV_SRDFR, FV_RDF, FV_KBRDF,
    FV_SHELL, FV_NVEC
};
enum FinalScalar {
    FS_TOTAL = 0, FS_BULK, FS_DOMAIN, FS_DSOLUTE, FS_DSOLVENT, FS_DSOLVENT_BULK, FS_DENSITY_FIX, FS_ZERO_RANDOM_BINS,
    FS_NSCALAR
};

struct FinalJob {
    const unsigned long long *acc;  // int64 half-unit counts of the open weight class
    const double *sums;             // folded weighted sums
    double class_w;
    int class_open;
    int nbins, Gs, Gv;              // Gv = 0 in self mode
    int autocorrelation, mddf_mode, usecutoff;
    int64_t o_md, o_mdr, o_rdf, o_rdfr, o_gs, o_gsr, o_gv, o_gvr;
    double binstep, dbulk;
    double Q;                       // sum of the frame weights (sum_frame_weights, src/results.jl:288-297)
    double volume_sum;              // sum of w * det(cell) over the frames (src/mddf.jl:352)
    double solute_nmols, solvent_nmols;
    double solvent_nmols_samples;   // set_samples (src/results.jl:230-237): nmols, or nmols - 1 in self mode
    double nrandom;
    double units_f;                 // units.Angs3tocm3permol (src/io.jl:6-14)
    int ibulk;                      // setbin(dbulk + binstep / 2, binstep), 1-based
    double *out;                    // packed output
};

__device__ __forceinline__ double final_weighted(const FinalJob &J, int64_t i) {
    const unsigned long long c = J.acc[i];
    // the host read-out's expression (cm_read_counts)
    return (J.class_open && c) ? add(J.sums[i], mul(J.class_w, div((double)c, 2.0))) : J.sums[i];
}

__global__ void k_finalize(const FinalJob *__restrict__ jobs) {
    const FinalJob J = jobs[blockIdx.x];
    const int nb = J.nbins;
    double *V = J.out;
    auto vec = [&](int k) { return V + (int64_t)k * nb; };
    double *gs = V + (int64_t)FV_NVEC * nb;
    double *gsr = gs + (int64_t)J.Gs * nb;
    double *gv = gsr + (int64_t)J.Gs * nb;
    const int Gv = J.autocorrelation ? J.Gs : J.Gv;
    double *gvr = gv + (int64_t)Gv * nb;
    double *sc = gvr + (int64_t)Gv * nb;
    const double nQ = mul(J.solute_nmols, J.Q), rQ = mul(J.nrandom, J.Q);
    const bool m = J.mddf_mode != 0;

    // normalisation by the frames and molecules (src/results.jl:322-337, 436-447)
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        const double rmin = mul((double)i, J.binstep), rmax = add(rmin, J.binstep);
        vec(FV_D)[i] = pow(mul(0.5, add(pow(rmax, 3.0), pow(rmin, 3.0))), 1.0 / 3.0);  // shellradius
        vec(FV_MD)[i] = div(final_weighted(J, J.o_md + i), nQ);
        vec(FV_RDFC)[i] = div(final_weighted(J, J.o_rdf + i), nQ);
        vec(FV_MDR)[i] = m ? div(final_weighted(J, J.o_mdr + i), rQ) : final_weighted(J, J.o_mdr + i);
        vec(FV_RDFCR)[i] = m ? div(final_weighted(J, J.o_rdfr + i), rQ) : final_weighted(J, J.o_rdfr + i);
    }
    for (int64_t i = threadIdx.x; i < (int64_t)J.Gs * nb; i += blockDim.x) {
        gs[i] = div(final_weighted(J, J.o_gs + i), nQ);
        gsr[i] = m ? div(final_weighted(J, J.o_gsr + i), rQ) : final_weighted(J, J.o_gsr + i);
        if (J.autocorrelation) {
            gv[i] = gs[i];
            gvr[i] = gsr[i];
        }
    }
    if (!J.autocorrelation)
        for (int64_t i = threadIdx.x; i < (int64_t)J.Gv * nb; i += blockDim.x) {
            gv[i] = div(final_weighted(J, J.o_gv + i), nQ);
            gvr[i] = m ? div(final_weighted(J, J.o_gvr + i), rQ) : final_weighted(J, J.o_gvr + i);
        }
    const double total = div(J.volume_sum, J.Q);
    if (m)
        for (int i = threadIdx.x; i < nb; i += blockDim.x)
            vec(FV_SHELL)[i] = mul(total, div(vec(FV_RDFCR)[i], J.solvent_nmols_samples));
    else
        for (int i = threadIdx.x; i < nb; i += blockDim.x) vec(FV_SHELL)[i] = 0.0;
    __syncthreads();

    // volumes and densities (src/results.jl:339-357), one thread, index order
    __shared__ double s_fix;
    if (threadIdx.x == 0) {
        for (int k = 0; k < FS_NSCALAR; ++k) sc[k] = 0.0;
        sc[FS_TOTAL] = total;
        sc[FS_DSOLVENT] = div(J.solvent_nmols, total);
        sc[FS_DSOLUTE] = div(J.solute_nmols, total);
        s_fix = 1.0;
        if (m) {
            const double *shell = vec(FV_SHELL), *rc = vec(FV_RDFC);
            double domain = 0.0;
            for (int i = 0; i < J.ibulk - 1 && i < nb; ++i) domain = i == 0 ? shell[i] : add(domain, shell[i]);
            double bulk, nbulk;
            if (!J.usecutoff) {
                bulk = sub(total, domain);
                double s = 0.0;
                for (int i = 0; i < nb; ++i) s = i == 0 ? rc[i] : add(s, rc[i]);
                nbulk = sub(J.solvent_nmols_samples, s);
            } else {
                double s = 0.0, b = 0.0;
                for (int i = J.ibulk - 1, k = 0; i < nb; ++i, ++k) {
                    s = k == 0 ? rc[i] : add(s, rc[i]);
                    b = k == 0 ? shell[i] : add(b, shell[i]);
                }
                nbulk = s;
                bulk = b;
            }
            sc[FS_DOMAIN] = domain;
            sc[FS_BULK] = bulk;
            sc[FS_DSOLVENT_BULK] = div(nbulk, bulk);
            s_fix = div(sc[FS_DSOLVENT_BULK], sc[FS_DSOLVENT]);
            sc[FS_DENSITY_FIX] = s_fix;
        }
    }
    __syncthreads();
    const double fix = s_fix;

    // renormalize! (src/results.jl:378-428)
    if (m) {
        for (int i = threadIdx.x; i < nb; i += blockDim.x) {
            vec(FV_MDR)[i] = mul(vec(FV_MDR)[i], fix);
            vec(FV_RDFCR)[i] = mul(vec(FV_RDFCR)[i], fix);
        }
        for (int64_t i = threadIdx.x; i < (int64_t)J.Gs * nb; i += blockDim.x) gsr[i] = mul(gsr[i], fix);
        for (int64_t i = threadIdx.x; i < (int64_t)Gv * nb; i += blockDim.x) gvr[i] = mul(gvr[i], fix);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double *md = vec(FV_MD), *mdr = vec(FV_MDR), *rc = vec(FV_RDFC), *rcr = vec(FV_RDFCR);
        double *cn = vec(FV_CN), *cnr = vec(FV_CNR), *srdf = vec(FV_SRDF), *srdfr = vec(FV_SRDFR);
        for (int i = 0; i < nb; ++i) {
            cn[i] = i == 0 ? md[i] : add(cn[i - 1], md[i]);
            srdf[i] = i == 0 ? rc[i] : add(srdf[i - 1], rc[i]);
            cnr[i] = m ? (i == 0 ? mdr[i] : add(cnr[i - 1], mdr[i])) : 0.0;
            srdfr[i] = m ? (i == 0 ? rcr[i] : add(srdfr[i - 1], rcr[i])) : 0.0;
        }
    }
    __syncthreads();
    int zero_bins = 0;
    if (m) {
        const double inv = div(1.0, sc[FS_DSOLVENT_BULK]);
        const double fi = mul(J.units_f, inv);
        for (int i = threadIdx.x; i < nb; i += blockDim.x) {
            const double mdr = vec(FV_MDR)[i], rcr = vec(FV_RDFCR)[i];
            vec(FV_MDDF)[i] = mdr > 0.0 ? div(vec(FV_MD)[i], mdr) : 0.0;
            zero_bins += mdr > 0.0 ? 0 : 1;
            vec(FV_KB)[i] = mul(fi, sub(vec(FV_CN)[i], vec(FV_CNR)[i]));
            vec(FV_RDF)[i] = rcr > 0.0 ? div(vec(FV_RDFC)[i], rcr) : 0.0;
            vec(FV_KBRDF)[i] = mul(fi, sub(vec(FV_SRDF)[i], vec(FV_SRDFR)[i]));
        }
    } else {
        for (int i = threadIdx.x; i < nb; i += blockDim.x)
            vec(FV_MDDF)[i] = vec(FV_KB)[i] = vec(FV_RDF)[i] = vec(FV_KBRDF)[i] = 0.0;
    }
    __shared__ int s_zero;
    if (threadIdx.x == 0) s_zero = 0;
    __syncthreads();
    if (zero_bins) atomicAdd(&s_zero, zero_bins);
    __syncthreads();
    if (threadIdx.x == 0) sc[FS_ZERO_RANDOM_BINS] = (double)s_zero;
}

// Contribution queries (contributions, src/tools/contributions.jl:70-248) on
// the packed output of k_finalize.  A query sums group-count rows of one side
// in the order of its terms (sel_count .+= group_count[g], or
// group_count[g] / nmols when the query names atoms of a multi-molecule
// selection), then converts the sum as the reference does for its type.
// ResidueContributions (src/tools/residue_contributions.jl:157-215) is one
// query per residue, so a whole protein is one launch.
enum ContribType { CT_MDDF = 0, CT_COORDINATION_NUMBER = 1, CT_MD_COUNT = 2, CT_KBI = 3 };

struct ContribQuery {
    int side;      // 0: solute groups, 1: solvent groups
    int type;      // ContribType
    int divide;    // terms are group_count[g] / nmols
    int t0, t1;    // terms [t0, t1) of the group list
    double nmols;  // molecules of the side's selection
};

struct ContribJob {
    const double *fin;    // k_finalize output of the handle
    int nbins, Gs, Gv;    // Gv = Gs in self mode (the solvent rows are the solute's)
    double units_f;       // units.Angs3tocm3permol (src/io.jl:6-14)
    const ContribQuery *q;
    const int *groups;
    double *out;          // [queries][nbins]
    double *scratch;      // [queries][nbins]: the random-count sums of KBI queries
};

__global__ void k_contrib(ContribJob J) {
    const ContribQuery Q = J.q[blockIdx.x];
    const int nb = J.nbins;
    const double *fin = J.fin;
    const double *mdr = fin + (int64_t)FV_MDR * nb;
    const double *gs = fin + (int64_t)FV_NVEC * nb;
    const double *gsr = gs + (int64_t)J.Gs * nb;
    const double *gv = gsr + (int64_t)J.Gs * nb;
    const double *gvr = gv + (int64_t)J.Gv * nb;
    const double *sc = gvr + (int64_t)J.Gv * nb;
    const double *gc = Q.side ? gv : gs, *gcr = Q.side ? gvr : gsr;
    double *out = J.out + (int64_t)blockIdx.x * nb;
    double *selr_out = J.scratch + (int64_t)blockIdx.x * nb;
    const bool kbi = Q.type == CT_KBI;
    // sel_count and sel_count_random, bin by bin, terms in order
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        double sel = 0.0, selr = 0.0;
        for (int t = Q.t0; t < Q.t1; ++t) {
            const int64_t row = (int64_t)J.groups[t] * nb + i;
            const double x = Q.divide ? div(gc[row], Q.nmols) : gc[row];
            sel = add(sel, x);
            if (kbi) selr = add(selr, Q.divide ? div(gcr[row], Q.nmols) : gcr[row]);
        }
        if (Q.type == CT_MDDF) sel = mdr[i] == 0.0 ? 0.0 : div(sel, mdr[i]);
        out[i] = sel;
        if (kbi) selr_out[i] = selr;
    }
    if (Q.type != CT_COORDINATION_NUMBER && !kbi) return;
    __syncthreads();
    if (threadIdx.x != 0) return;
    // cumulative sums in index order (cumsum), then the KBI expression
    double c = 0.0, cr = 0.0;
    const double fi = kbi ? mul(J.units_f, div(1.0, sc[FS_DSOLVENT_BULK])) : 0.0;
    for (int i = 0; i < nb; ++i) {
        c = i == 0 ? out[i] : add(c, out[i]);
        if (kbi) {
            cr = i == 0 ? selr_out[i] : add(cr, selr_out[i]);
            out[i] = mul(fi, sub(c, cr));
        } else {
            out[i] = c;
        }
    }
}

}  // namespace cmk
