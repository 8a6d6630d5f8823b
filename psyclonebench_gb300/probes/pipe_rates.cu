// Issue-rate probe: FP64 FMA/MUL/ADD/DIV/SQRT, FP32 FMA and integer rates
// with 8 independent chains per thread over 8 CTAs per SM, and a double2
// copy for HBM bandwidth; the numbers decide which roof bounds each form of
// the NEMOLite2D step on this GPU.
#include <cstdio>
#include <cuda_runtime.h>

#include "../csrc/nl2d_intfp.cuh"
using nl2d::dadd_i;
using nl2d::dmul_i;
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n",cudaGetErrorString(e),__LINE__); return 1;}}while(0)

template<int OP>
__global__ void kdp(double* out, double a, double b, int iters){
  double x0=threadIdx.x*1e-3+1.0, x1=x0+0.1, x2=x0+0.2, x3=x0+0.3, x4=x0+0.4, x5=x0+0.5, x6=x0+0.6, x7=x0+0.7;
  for(int i=0;i<iters;i++){
    if(OP==0){ x0=fma(x0,a,b); x1=fma(x1,a,b); x2=fma(x2,a,b); x3=fma(x3,a,b); x4=fma(x4,a,b); x5=fma(x5,a,b); x6=fma(x6,a,b); x7=fma(x7,a,b);}
    if(OP==1){ x0=x0*a; x1=x1*a; x2=x2*a; x3=x3*a; x4=x4*a; x5=x5*a; x6=x6*a; x7=x7*a;}
    if(OP==2){ x0=x0+a; x1=x1+a; x2=x2+a; x3=x3+a; x4=x4+a; x5=x5+a; x6=x6+a; x7=x7+a;}
    if(OP==3){ x0=b/x0; x1=b/x1; x2=b/x2; x3=b/x3; x4=b/x4; x5=b/x5; x6=b/x6; x7=b/x7;}
    if(OP==4){ x0=sqrt(x0); x1=sqrt(x1); x2=sqrt(x2); x3=sqrt(x3); x4=sqrt(x4); x5=sqrt(x5); x6=sqrt(x6); x7=sqrt(x7);}
    // exact IEEE add / multiply on the integer pipes, and half of the
    // chains on each pipe (what the FP64 step can hope for when it splits)
    if(OP==5){ x0=dadd_i(x0,a); x1=dadd_i(x1,a); x2=dadd_i(x2,a); x3=dadd_i(x3,a); x4=dadd_i(x4,a); x5=dadd_i(x5,a); x6=dadd_i(x6,a); x7=dadd_i(x7,a);}
    if(OP==6){ x0=dmul_i(x0,a); x1=dmul_i(x1,a); x2=dmul_i(x2,a); x3=dmul_i(x3,a); x4=dmul_i(x4,a); x5=dmul_i(x5,a); x6=dmul_i(x6,a); x7=dmul_i(x7,a);}
    if(OP==7){ x0=x0+a; x1=x1+a; x2=x2+a; x3=x3+a; x4=dadd_i(x4,a); x5=dadd_i(x5,a); x6=dadd_i(x6,a); x7=dadd_i(x7,a);}
  }
  out[blockIdx.x*blockDim.x+threadIdx.x]=x0+x1+x2+x3+x4+x5+x6+x7;
}
__global__ void ksp(float* out, float a, float b, int iters){
  float x0=threadIdx.x*1e-3f+1.0f, x1=x0+0.1f, x2=x0+0.2f, x3=x0+0.3f, x4=x0+0.4f, x5=x0+0.5f, x6=x0+0.6f, x7=x0+0.7f;
  for(int i=0;i<iters;i++){ x0=fmaf(x0,a,b); x1=fmaf(x1,a,b); x2=fmaf(x2,a,b); x3=fmaf(x3,a,b); x4=fmaf(x4,a,b); x5=fmaf(x5,a,b); x6=fmaf(x6,a,b); x7=fmaf(x7,a,b);}
  out[blockIdx.x*blockDim.x+threadIdx.x]=x0+x1+x2+x3+x4+x5+x6+x7;
}
__global__ void kint(unsigned* out, unsigned a, unsigned b, int iters){
  unsigned x0=threadIdx.x, x1=x0+1, x2=x0+2, x3=x0+3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for(int i=0;i<iters;i++){ x0=x0*a+b; x1=x1*a+b; x2=x2*a+b; x3=x3*a+b; x4=x4*a+b; x5=x5*a+b; x6=x6*a+b; x7=x7*a+b;}
  out[blockIdx.x*blockDim.x+threadIdx.x]=x0^x1^x2^x3^x4^x5^x6^x7;
}
__global__ void kiadd(unsigned* out, unsigned a, unsigned b, int iters){
  unsigned x0=threadIdx.x, x1=x0+1, x2=x0+2, x3=x0+3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for(int i=0;i<iters;i++){ x0=(x0^a)+b; x1=(x1^a)+b; x2=(x2^a)+b; x3=(x3^a)+b; x4=(x4^a)+b; x5=(x5^a)+b; x6=(x6^a)+b; x7=(x7^a)+b;}
  out[blockIdx.x*blockDim.x+threadIdx.x]=x0^x1^x2^x3^x4^x5^x6^x7;
}
// 64-bit integer add + shift chains: do they run on the 32-bit integer
// pipes (as pairs) or share the FP64 pipe?
__global__ void kint64(unsigned long long* out, unsigned long long a, int iters){
  unsigned long long x0=threadIdx.x, x1=x0+1, x2=x0+2, x3=x0+3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for(int i=0;i<iters;i++){
    x0=(x0+a)^(x0>>11); x1=(x1+a)^(x1>>11); x2=(x2+a)^(x2>>11); x3=(x3+a)^(x3>>11);
    x4=(x4+a)^(x4>>11); x5=(x5+a)^(x5>>11); x6=(x6+a)^(x6>>11); x7=(x7+a)^(x7>>11);
  }
  out[blockIdx.x*blockDim.x+threadIdx.x]=x0^x1^x2^x3^x4^x5^x6^x7;
}

__global__ void kcopy(const double2* __restrict__ a, double2* __restrict__ b, size_t n){
  size_t i=blockIdx.x*(size_t)blockDim.x+threadIdx.x, s=(size_t)gridDim.x*blockDim.x;
  for(;i<n;i+=s) b[i]=a[i];
}
int main(){
  int nb=152*8, nt=256, iters=4096;
  double* od; float* of; unsigned* oi;
  CK(cudaMalloc(&od, nb*nt*8)); CK(cudaMalloc(&of, nb*nt*4)); CK(cudaMalloc(&oi, nb*nt*4));
  cudaEvent_t e0,e1; cudaEventCreate(&e0); cudaEventCreate(&e1); float ms;
  const char* names[8]={"DFMA","DMUL","DADD","DDIV","DSQRT","dadd_i (integer pipes)","dmul_i (integer pipes)","4 DADD + 4 dadd_i chains"};
  for(int rep=0;rep<2;rep++){
  for(int op=0;op<8;op++){
    int it = (op>=3)? iters/8: iters;
    auto launch=[&](){ if(op==0) kdp<0><<<nb,nt>>>(od,1.0000001,1e-9,it); if(op==1) kdp<1><<<nb,nt>>>(od,1.0000001,0,it);
      if(op==2) kdp<2><<<nb,nt>>>(od,1e-9,0,it); if(op==3) kdp<3><<<nb,nt>>>(od,0,1.0000001,it); if(op==4) kdp<4><<<nb,nt>>>(od,0,0,it);
      if(op==5) kdp<5><<<nb,nt>>>(od,1e-9,0,it); if(op==6) kdp<6><<<nb,nt>>>(od,1.0000001,0,it); if(op==7) kdp<7><<<nb,nt>>>(od,1e-9,0,it);};
    launch(); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); launch(); cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms,e0,e1);
    double nops=(double)nb*nt*it*8;
    printf("%s: %.3f ms, %.1f Gop/s, %.3f op/clk/SM@1.9GHz\n", names[op], ms, nops/ms/1e6, nops/(ms*1e-3)/152/1.9e9);
  }
  {
    ksp<<<nb,nt>>>(of,1.0000001f,1e-9f,iters*8); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); ksp<<<nb,nt>>>(of,1.0000001f,1e-9f,iters*8); cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms,e0,e1);
    double nops=(double)nb*nt*iters*8*8; printf("FFMA: %.3f ms, %.1f Gop/s, %.2f op/clk/SM\n", ms, nops/ms/1e6, nops/(ms*1e-3)/152/1.9e9);
    kint<<<nb,nt>>>(oi,12345u,7u,iters*8); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); kint<<<nb,nt>>>(oi,12345u,7u,iters*8); cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms,e0,e1);
    printf("IMAD: %.3f ms, %.1f Gop/s, %.2f op/clk/SM\n", ms, nops/ms/1e6, nops/(ms*1e-3)/152/1.9e9);
    kiadd<<<nb,nt>>>(oi,12345u,7u,iters*8); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); kiadd<<<nb,nt>>>(oi,12345u,7u,iters*8); cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms,e0,e1);
    printf("LOP3+IADD pairs: %.3f ms, %.1f Gpair/s, %.2f pair/clk/SM\n", ms, nops/ms/1e6, nops/(ms*1e-3)/152/1.9e9);
  }
  {
    unsigned long long* o64; CK(cudaMalloc(&o64, nb*nt*8));
    kint64<<<nb,nt>>>(o64,0x9E3779B97F4A7C15ULL,iters); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); kint64<<<nb,nt>>>(o64,0x9E3779B97F4A7C15ULL,iters); cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms,e0,e1);
    double nops=(double)nb*nt*iters*8;
    printf("64-bit add+shift+xor steps: %.3f ms, %.1f Gstep/s, %.2f step/clk/SM\n", ms, nops/ms/1e6, nops/(ms*1e-3)/152/1.9e9);
    cudaFree(o64);
  }
  }
  size_t n=(size_t)1<<27; double2 *a,*b; CK(cudaMalloc(&a,n*16)); CK(cudaMalloc(&b,n*16)); cudaMemset(a,0,n*16);
  for(int r=0;r<3;r++){ cudaEventRecord(e0); kcopy<<<152*16,256>>>(a,b,n); cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); cudaEventElapsedTime(&ms,e0,e1);
    printf("copy 2x%.1f GB: %.3f ms, %.1f GB/s\n", n*16/1e9, ms, 2.0*n*16/ms/1e6); }
  int dev; cudaGetDevice(&dev); cudaDeviceProp p; cudaGetDeviceProperties(&p,dev);
  printf("%s SMs=%d smem/blk optin=%zu L2=%d\n", p.name, p.multiProcessorCount, p.sharedMemPerBlockOptin, p.l2CacheSize);
  return 0;
}
