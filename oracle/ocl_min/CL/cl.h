/* Minimal OpenCL 2.0 host declarations for building the reference program
 * (mersenne2_gpu.cpp) where no OpenCL headers are installed.  Written for this
 * repository from the public OpenCL API specification: only the types,
 * constants and entry points that program calls.  oracle/ocl_min/icd_min.cpp
 * defines the entry points.  Test infrastructure: only the reference-timing
 * recipe (oracle/build_ref.py) uses it. */
#ifndef M2_OCL_MIN_CL_H
#define M2_OCL_MIN_CL_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CL_API_CALL
#define CL_CALLBACK

typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef uint64_t cl_ulong;
typedef cl_ulong cl_bitfield;
typedef cl_uint cl_bool;
typedef cl_bitfield cl_device_type;
typedef cl_uint cl_platform_info;
typedef cl_uint cl_device_info;
typedef cl_bitfield cl_mem_flags;
typedef cl_uint cl_program_build_info;
typedef cl_bitfield cl_command_queue_properties;
typedef cl_bitfield cl_queue_properties;
typedef intptr_t cl_context_properties;

typedef struct _cl_platform_id* cl_platform_id;
typedef struct _cl_device_id* cl_device_id;
typedef struct _cl_context* cl_context;
typedef struct _cl_command_queue* cl_command_queue;
typedef struct _cl_mem* cl_mem;
typedef struct _cl_program* cl_program;
typedef struct _cl_kernel* cl_kernel;
typedef struct _cl_event* cl_event;

#define CL_SUCCESS 0
#define CL_DEVICE_NOT_FOUND -1
#define CL_INVALID_VALUE -30
#define CL_PLATFORM_NOT_FOUND_KHR -1001
#define CL_FALSE 0
#define CL_TRUE 1

#define CL_PLATFORM_NAME 0x0902
#define CL_DEVICE_TYPE_GPU (1 << 2)
#define CL_DEVICE_MAX_COMPUTE_UNITS 0x1002
#define CL_DEVICE_MAX_WORK_GROUP_SIZE 0x1004
#define CL_DEVICE_LOCAL_MEM_SIZE 0x1023
#define CL_DEVICE_NAME 0x102B
#define CL_DEVICE_VENDOR 0x102C

#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_READ_ONLY (1 << 2)
#define CL_MEM_COPY_HOST_PTR (1 << 5)

#define CL_PROGRAM_BUILD_LOG 0x1183

cl_int clGetPlatformIDs(cl_uint num_entries, cl_platform_id* platforms, cl_uint* num_platforms);
cl_int clGetDeviceIDs(cl_platform_id platform, cl_device_type device_type, cl_uint num_entries, cl_device_id* devices,
                      cl_uint* num_devices);
cl_int clGetDeviceInfo(cl_device_id device, cl_device_info param_name, size_t param_value_size, void* param_value,
                       size_t* param_value_size_ret);
cl_context clCreateContext(const cl_context_properties* properties, cl_uint num_devices, const cl_device_id* devices,
                           void(CL_CALLBACK* pfn_notify)(const char*, const void*, size_t, void*), void* user_data,
                           cl_int* errcode_ret);
cl_command_queue clCreateCommandQueue(cl_context context, cl_device_id device, cl_command_queue_properties properties,
                                      cl_int* errcode_ret);
cl_command_queue clCreateCommandQueueWithProperties(cl_context context, cl_device_id device,
                                                    const cl_queue_properties* properties, cl_int* errcode_ret);
cl_program clCreateProgramWithSource(cl_context context, cl_uint count, const char** strings, const size_t* lengths,
                                     cl_int* errcode_ret);
cl_int clBuildProgram(cl_program program, cl_uint num_devices, const cl_device_id* device_list, const char* options,
                      void(CL_CALLBACK* pfn_notify)(cl_program, void*), void* user_data);
cl_int clGetProgramBuildInfo(cl_program program, cl_device_id device, cl_program_build_info param_name,
                             size_t param_value_size, void* param_value, size_t* param_value_size_ret);
cl_kernel clCreateKernel(cl_program program, const char* kernel_name, cl_int* errcode_ret);
cl_int clSetKernelArg(cl_kernel kernel, cl_uint arg_index, size_t arg_size, const void* arg_value);
cl_mem clCreateBuffer(cl_context context, cl_mem_flags flags, size_t size, void* host_ptr, cl_int* errcode_ret);
cl_int clEnqueueNDRangeKernel(cl_command_queue queue, cl_kernel kernel, cl_uint work_dim, const size_t* global_work_offset,
                              const size_t* global_work_size, const size_t* local_work_size,
                              cl_uint num_events_in_wait_list, const cl_event* event_wait_list, cl_event* event);
cl_int clEnqueueReadBuffer(cl_command_queue queue, cl_mem buffer, cl_bool blocking_read, size_t offset, size_t size,
                           void* ptr, cl_uint num_events_in_wait_list, const cl_event* event_wait_list, cl_event* event);
cl_int clFinish(cl_command_queue queue);
cl_int clReleaseKernel(cl_kernel kernel);
cl_int clReleaseMemObject(cl_mem memobj);
cl_int clReleaseProgram(cl_program program);
cl_int clReleaseCommandQueue(cl_command_queue queue);
cl_int clReleaseContext(cl_context context);

#ifdef __cplusplus
}
#endif
#endif
