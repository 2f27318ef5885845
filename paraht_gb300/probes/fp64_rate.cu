// Microbenchmark: FP64/FP32 throughput and dependent-instruction latency, FP64 shuffle-reduction
// latency and DMMA (mma.sync f64) throughput on one GPU.  These numbers set the FP64 roofline of
// the plain path and explain why the small serial factorizations are latency-bound.
// Build and run: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fp64_rate fp64_rate.cu && ./fp64_rate
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("ERR %s @%d: %s\n",#x,__LINE__,cudaGetErrorString(e)); return 1;}}while(0)

template<typename T>
__global__ void thr(T* out, int iters, T a, T b){
  T x0=threadIdx.x, x1=x0+1, x2=x0+2, x3=x0+3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for(int i=0;i<iters;i++){
    x0=x0*a+b; x1=x1*a+b; x2=x2*a+b; x3=x3*a+b; x4=x4*a+b; x5=x5*a+b; x6=x6*a+b; x7=x7*a+b;
  }
  out[blockIdx.x*blockDim.x+threadIdx.x]=x0+x1+x2+x3+x4+x5+x6+x7;
}
// dependent chain latency, active lanes = nact
__global__ void lat(double* out, long long* cyc, int iters, double a, double b, int nact){
  double x=threadIdx.x;
  long long t0=clock64();
  if(threadIdx.x<nact){
    for(int i=0;i<iters;i++){ x=x*a+b; }
  }
  long long t1=clock64();
  out[threadIdx.x]=x;
  if(threadIdx.x==0) cyc[blockIdx.x]=t1-t0;
}
__global__ void latf(float* out, long long* cyc, int iters, float a, float b){
  float x=threadIdx.x;
  long long t0=clock64();
  for(int i=0;i<iters;i++){ x=x*a+b; }
  long long t1=clock64();
  out[threadIdx.x]=x;
  if(threadIdx.x==0) cyc[blockIdx.x]=t1-t0;
}
// shuffle reduction latency in fp64
__global__ void shfl_red(double* out, long long* cyc, int iters){
  double x=threadIdx.x*1e-3;
  long long t0=clock64();
  for(int i=0;i<iters;i++){
    for(int o=16;o>0;o>>=1) x+=__shfl_xor_sync(0xffffffff,x,o);
    x*=1e-6;
  }
  long long t1=clock64();
  out[threadIdx.x]=x;
  if(threadIdx.x==0) cyc[0]=t1-t0;
}
// DMMA m8n8k4 throughput
__global__ void dmma(double* out, int iters){
  double a=threadIdx.x*1e-3, b=1.0001;
  double c0=0,c1=0, d0=0,d1=0, e0=0,e1=0, f0=0,f1=0;
  for(int i=0;i<iters;i++){
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};" : "+d"(c0),"+d"(c1) : "d"(a),"d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};" : "+d"(d0),"+d"(d1) : "d"(a),"d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};" : "+d"(e0),"+d"(e1) : "d"(a),"d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1},{%2},{%3},{%0,%1};" : "+d"(f0),"+d"(f1) : "d"(a),"d"(b));
  }
  out[blockIdx.x*blockDim.x+threadIdx.x]=c0+c1+d0+d1+e0+e1+f0+f1;
}
int main(){
  int dev=0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p,dev));
  int clk=0; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);
  printf("name %s SMs %d clockKHz %d smemOptin %zu L2 %d\n", p.name, p.multiProcessorCount, clk, p.sharedMemPerBlockOptin, p.l2CacheSize);
  int nsm=p.multiProcessorCount;
  double* d; CK(cudaMalloc(&d, 64ull<<20)); long long* cyc; CK(cudaMalloc(&cyc, 4096*8));
  cudaEvent_t e0,e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  // throughput fp64
  for(int rep=0;rep<2;rep++){
    int blocks=nsm*8, threads=256, iters=4096;
    cudaEventRecord(e0); thr<double><<<blocks,threads>>>(d,iters,1.0000001,1e-9); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms,e0,e1);
    double fl=2.0*8*iters*(double)blocks*threads;
    printf("fp64 FMA throughput: %.3f TFLOP/s (%.3f ms)\n", fl/ms/1e9, ms);
  }
  for(int rep=0;rep<2;rep++){
    int blocks=nsm*8, threads=256, iters=65536;
    cudaEventRecord(e0); thr<float><<<blocks,threads>>>((float*)d,iters,1.0000001f,1e-9f); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms,e0,e1);
    double fl=2.0*8*iters*(double)blocks*threads;
    printf("fp32 FMA throughput: %.3f TFLOP/s (%.3f ms)\n", fl/ms/1e9, ms);
  }
  // single SM fp64 throughput with varying warps
  for(int w=1; w<=32; w*=2){
    int iters=2048;
    cudaEventRecord(e0); thr<double><<<1,32*w>>>(d,iters,1.0000001,1e-9); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms,e0,e1);
    double fma=8.0*iters*32*w;
    printf("1 SM fp64: warps %2d  %.2f FMA/ns (%.3f ms)\n", w, fma/ms/1e6, ms);
  }
  // latency
  long long h[4];
  for(int nact: {32, 8, 1}){
    lat<<<1,32>>>(d,cyc,1024,1.0000001,1e-9,nact); CK(cudaDeviceSynchronize());
    lat<<<1,32>>>(d,cyc,1024,1.0000001,1e-9,nact); CK(cudaDeviceSynchronize());
    cudaMemcpy(h,cyc,8,cudaMemcpyDeviceToHost);
    printf("fp64 dep-chain 1 warp (%d lanes active): %.1f clk/FMA\n", nact, h[0]/1024.0);
  }
  for(int wb: {4, 8, 16}){
    lat<<<1,32*wb>>>(d,cyc,1024,1.0000001,1e-9,32*wb); CK(cudaDeviceSynchronize());
    cudaMemcpy(h,cyc,8,cudaMemcpyDeviceToHost);
    printf("fp64 dep-chain %d warps in 1 CTA: %.1f clk/FMA (warp0)\n", wb, h[0]/1024.0);
  }
  latf<<<1,32>>>((float*)d,cyc,1024,1.0000001f,1e-9f); CK(cudaDeviceSynchronize());
  cudaMemcpy(h,cyc,8,cudaMemcpyDeviceToHost); printf("fp32 dep-chain: %.1f clk/FMA\n", h[0]/1024.0);
  shfl_red<<<1,32>>>(d,cyc,256); CK(cudaDeviceSynchronize());
  cudaMemcpy(h,cyc,8,cudaMemcpyDeviceToHost); printf("fp64 5-step shfl reduction: %.1f clk each\n", h[0]/256.0);
  // DMMA
  for(int rep=0;rep<2;rep++){
    int blocks=nsm*4, threads=256, iters=2048;
    cudaEventRecord(e0); dmma<<<blocks,threads>>>(d,iters); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms,e0,e1);
    double fl=2.0*8*8*4*4.0*iters*(double)blocks*threads/32;
    printf("DMMA m8n8k4 throughput: %.3f TFLOP/s (%.3f ms)\n", fl/ms/1e9, ms);
  }
  CK(cudaGetLastError());
  return 0;
}
