// Operator preparation: once per set_operators call, in FP64, then rounded to
// the plan's working precision.
//
// The reference rebuilds L^dag L and the anticommutator inside every RHS call
// (pyqed/oqs.py:707-715).  Here H_eff = H - c I - (i/2) sum_k L_k^dag L_k is
// formed once (c = Re Tr(H)/N; shifting H by a multiple of the identity leaves
// -i[H, rho] unchanged and keeps the stored entries small, which matters for
// the reduced-precision paths), and the kernels get
//   At  = (-i H_eff)^T                       NP x NPS, zero padded
//   Lt  = L_k^T                              dense collapse operators
//   Dm  = sum_k l_k l_k^dag (entrywise)      diagonal collapse operators
//   Gt  = (i H_d)^T                          drive terms (H(t) = H0 - f H_d)
//   Ot  = O_e^T (FP64)                       observables
#include <algorithm>

#include "lgb_internal.h"

namespace lgb {

namespace {

__global__ void trace_shift_kernel(SetupParams p) {
  const int b = blockIdx.x;
  const int N = p.dims[b];
  const double2* H = p.H + p.off[b];
  double s = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) s += H[(long long)i * N + i].x;
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) p.shift[b] = red[0] / (double)N;
}

template <typename T>
__global__ void setup_kernel(SetupParams p) {
  using T2 = typename Cplx<T>::type;
  const int b = blockIdx.y;
  const int N = p.dims[b];
  const int NP = p.npad[b];
  const int NPS = NP + p.padc;
  const long long MS = (long long)NP * NPS;
  const long long wo = p.woff[b];
  const long long o = p.off[b];
  const long long NN = (long long)N * N;
  const int K = p.n_cops;
  const double c = p.shift[b];
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < MS;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / NPS);  // row of the stored (transposed) matrix
    const int q = (int)(idx % NPS);  // column of the stored matrix
    const bool in = (r < N) && (q < N);
    // At[r][q] = A[q][r], A = -i (H - c I) - G/2
    {
      double2 a = make_double2(0.0, 0.0);
      if (in) {
        const double2 h = p.H[o + (long long)q * N + r];
        double hx = h.x - ((q == r) ? c : 0.0);
        a = make_double2(h.y, -hx);  // -i * (hx + i hy) = hy - i hx
        double gx = 0.0, gy = 0.0;
        if (p.cops_kind == 1) {
          // G[q][r] = sum_k sum_m conj(L_k[m][q]) L_k[m][r]
          for (int k = 0; k < K; ++k) {
            const double2* L = p.cops + (long long)K * o + k * NN;
            for (int m = 0; m < N; ++m) {
              const double2 u = L[(long long)m * N + q];
              const double2 v = L[(long long)m * N + r];
              gx += u.x * v.x + u.y * v.y;
              gy += u.x * v.y - u.y * v.x;
            }
          }
        } else if (p.cops_kind == 2 && q == r) {
          for (int k = 0; k < K; ++k) {
            const double2 l = p.cops[(long long)K * p.doff[b] + (long long)k * N + q];
            gx += l.x * l.x + l.y * l.y;
          }
        }
        a.x -= 0.5 * gx;
        a.y -= 0.5 * gy;
      }
      reinterpret_cast<T2*>(p.At)[wo + idx] = mk<T2>(a.x, a.y);
    }
    if (p.cops_kind == 1) {
      for (int k = 0; k < K; ++k) {
        double2 v = make_double2(0.0, 0.0);
        if (in) v = p.cops[(long long)K * o + k * NN + (long long)q * N + r];
        reinterpret_cast<T2*>(p.Lt)[(long long)K * wo + k * MS + idx] = mk<T2>(v.x, v.y);
      }
    } else if (p.cops_kind == 2) {
      // Dm[r][q] = sum_k l_k[r] conj(l_k[q])
      double dx = 0.0, dy = 0.0;
      if (in) {
        for (int k = 0; k < K; ++k) {
          const double2* l = p.cops + (long long)K * p.doff[b] + (long long)k * N;
          const double2 u = l[r], v = l[q];
          dx += u.x * v.x + u.y * v.y;
          dy += u.y * v.x - u.x * v.y;
        }
      }
      reinterpret_cast<T2*>(p.Dm)[wo + idx] = mk<T2>(dx, dy);
    }
    for (int d = 0; d < p.n_drive; ++d) {
      double2 g = make_double2(0.0, 0.0);
      if (in) {
        const double2 h = p.dops[(long long)p.n_drive * o + d * NN + (long long)q * N + r];
        g = make_double2(-h.y, h.x);  // i * h
      }
      reinterpret_cast<T2*>(p.Gt)[(long long)p.n_drive * wo + d * MS + idx] = mk<T2>(g.x, g.y);
    }
    for (int e = 0; e < p.n_eops; ++e) {
      double2 v = make_double2(0.0, 0.0);
      if (in) v = p.eops[(long long)p.n_eops * o + e * NN + (long long)q * N + r];
      p.Ot[(long long)p.n_eops * wo + e * MS + idx] = v;
      if (p.OtF != nullptr)
        p.OtF[(long long)p.n_eops * wo + e * MS + idx] = make_float2((float)v.x, (float)v.y);
    }
  }
}

}  // namespace

cudaError_t launch_trace_shift(const SetupParams& p, cudaStream_t stream) {
  trace_shift_kernel<<<p.n_inst, 256, 0, stream>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_setup(const SetupParams& p, int precision, cudaStream_t stream) {
  trace_shift_kernel<<<p.n_inst, 256, 0, stream>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // blocks per instance: enough for the largest padded matrix, at most 64
  const long long ms = (long long)p.max_npad * (p.max_npad + p.padc);
  const int gx = (int)std::max<long long>(1, std::min<long long>(64, (ms + 255) / 256));
  dim3 grid(gx, p.n_inst);
  if (precision == 0) {
    setup_kernel<double><<<grid, 256, 0, stream>>>(p);
  } else {
    setup_kernel<float><<<grid, 256, 0, stream>>>(p);
  }
  return cudaGetLastError();
}

}  // namespace lgb
