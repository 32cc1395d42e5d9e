// vx3g_adjoint.cu -- kernels of the FP64 adjoint (per-element math in vx3g_adjoint.cuh)
// and the state-snapshot copy used by the recorded run and its recomputation.
#include "vx3g_adjoint.cuh"

namespace vx3g {

__global__ void __launch_bounds__(256) k_snap_copy(Snap dst, Snap src, int nv, int nl, int nr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) {
        dst.pos[i] = src.pos[i];
        dst.quat[i] = src.quat[i];
        dst.linmom[i] = src.linmom[i];
        dst.angmom[i] = src.angmom[i];
        dst.vinfo[i] = src.vinfo[i];
        dst.tempe[i] = src.tempe[i];
        dst.tempe[nv + i] = src.tempe[nv + i];
    }
    if (i < nl) {
        for (int k = 0; k < 9; k++) dst.lstate[(size_t)k * nl + i] = src.lstate[(size_t)k * nl + i];
        dst.strain[i] = src.strain[i];
        dst.linfo[i] = src.linfo[i];
    }
    if (i < nr) {
        dst.T[i] = src.T[i];
        dst.T[nr + i] = src.T[nr + i];
        dst.status[i] = src.status[i];
    }
}

void launch_snap_copy(const Snap &dst, const Snap &src, int nv, int nl, int nr, cudaStream_t st) {
    int n = nv > nl ? nv : nl;
    if (nr > n) n = nr;
    if (n) k_snap_copy<<<(n + 255) / 256, 256, 0, st>>>(dst, src, nv, nl, nr);
}

__global__ void __launch_bounds__(128) k_adj_slots(Dev d, Snap s, AdjBufs a) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < d.nl) adj::adj_link_slots(d, s, a, l);
}
// gather of step k+1 (state snapshot sg, parity a.parity) fused with the link-force
// recompute of step k (state snapshot ss): independent work, one launch
__global__ void __launch_bounds__(128) k_adj_gather_slots(Dev d, Snap sg, Snap ss, AdjBufs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.nv) adj::adj_gather(d, sg, a, i);
    if (i < d.nl) adj::adj_link_slots(d, ss, a, i);
}
__global__ void __launch_bounds__(128) k_adj_voxel(Dev d, Snap s, AdjBufs a) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < d.nv) adj::adj_voxel(d, s, a, v);
}
__global__ void __launch_bounds__(128) k_adj_link(Dev d, Snap s, AdjBufs a) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < d.nl) adj::adj_link(d, s, a, l);
}
__global__ void __launch_bounds__(128) k_adj_gather(Dev d, Snap s, AdjBufs a) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < d.nv) adj::adj_gather(d, s, a, v);
}
__global__ void __launch_bounds__(128) k_adj_seed(Dev d, AdjBufs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.nv) adj::adj_seed(d, a, i);
    if (i < d.nl)
        for (int k = 0; k < 9; k++) a.lloc[9 * (size_t)i + k] = 0.0;
}

void launch_adj_slots(const Dev &d, const Snap &s, const AdjBufs &a, cudaStream_t st) {
    if (d.nl) k_adj_slots<<<(d.nl + 127) / 128, 128, 0, st>>>(d, s, a);
}
void launch_adj_voxel_link(const Dev &d, const Snap &s, const AdjBufs &a, cudaStream_t st) {
    if (d.nv) k_adj_voxel<<<(d.nv + 127) / 128, 128, 0, st>>>(d, s, a);
    if (d.nl) k_adj_link<<<(d.nl + 127) / 128, 128, 0, st>>>(d, s, a);
}
void launch_adj_gather_slots(const Dev &d, const Snap &sg, const Snap *ss, const AdjBufs &a, cudaStream_t st) {
    const int n = d.nv > d.nl ? d.nv : d.nl;
    if (!ss) {
        if (d.nv) k_adj_gather<<<(d.nv + 127) / 128, 128, 0, st>>>(d, sg, a);
    } else if (n) {
        k_adj_gather_slots<<<(n + 127) / 128, 128, 0, st>>>(d, sg, *ss, a);
    }
}

__global__ void __launch_bounds__(128) k_adj_contact(Dev d, Snap s, AdjBufs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < d.ns) adj::adj_contact(d, s, a, i);
}

void launch_adj_contact(const Dev &d, const Snap &s, const AdjBufs &a, cudaStream_t st) {
    if (d.ns) k_adj_contact<<<(d.ns + 127) / 128, 128, 0, st>>>(d, s, a);
}

void launch_adj_seed(const Dev &d, const AdjBufs &a, cudaStream_t st) {
    const int n = d.nv > d.nl ? d.nv : d.nl;
    if (n) k_adj_seed<<<(n + 127) / 128, 128, 0, st>>>(d, a);
}

}  // namespace vx3g
