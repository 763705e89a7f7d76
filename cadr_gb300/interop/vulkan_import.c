/* vulkan_import.c - the Vulkan side of a cadr_shared_buffer: a renderer
 * imports the exported descriptor as the memory of an indirect-draw buffer
 * and draws the pass's commands from it with no copy (the importing half
 * of the reference's idiom, examples/OpenGLInteroperability/main.cpp:
 * 1488-1490 and 1616-1619, with Vulkan as the importer).
 *
 * Needs VK_KHR_external_memory_fd on the device.  `memory_type_index` must
 * be a device-local type allowed by vkGetMemoryFdPropertiesKHR for the
 * descriptor.  This file is compiled (syntax only) against the Vulkan
 * headers; it is not linked into the library, which has no Vulkan
 * dependency. */
#include <stdint.h>
#include <vulkan/vulkan_core.h>

#include "../../include/cadr_cuda.h"

/* Imports `fd` (from cadr_shared_buffer_export_fd; Vulkan takes ownership
 * of it on success) as a buffer of `size` bytes (cadr_shared_buffer_size)
 * usable as an indirect-draw and storage buffer. */
VkResult cadr_vk_import_shared_buffer(VkDevice device, int fd, VkDeviceSize size, uint32_t memory_type_index,
                                      VkBuffer* buffer, VkDeviceMemory* memory)
{
    const VkExternalMemoryBufferCreateInfo ext = {
        VK_STRUCTURE_TYPE_EXTERNAL_MEMORY_BUFFER_CREATE_INFO, NULL,
        VK_EXTERNAL_MEMORY_HANDLE_TYPE_OPAQUE_FD_BIT,
    };
    const VkBufferCreateInfo bci = {
        VK_STRUCTURE_TYPE_BUFFER_CREATE_INFO, &ext, 0, size,
        VK_BUFFER_USAGE_INDIRECT_BUFFER_BIT | VK_BUFFER_USAGE_STORAGE_BUFFER_BIT |
            VK_BUFFER_USAGE_SHADER_DEVICE_ADDRESS_BIT,
        VK_SHARING_MODE_EXCLUSIVE, 0, NULL,
    };
    VkResult r = vkCreateBuffer(device, &bci, NULL, buffer);
    if (r != VK_SUCCESS) return r;
    const VkImportMemoryFdInfoKHR import_info = {
        VK_STRUCTURE_TYPE_IMPORT_MEMORY_FD_INFO_KHR, NULL, VK_EXTERNAL_MEMORY_HANDLE_TYPE_OPAQUE_FD_BIT, fd,
    };
    const VkMemoryAllocateFlagsInfo flags = {
        VK_STRUCTURE_TYPE_MEMORY_ALLOCATE_FLAGS_INFO, &import_info, VK_MEMORY_ALLOCATE_DEVICE_ADDRESS_BIT, 0,
    };
    const VkMemoryAllocateInfo mai = {
        VK_STRUCTURE_TYPE_MEMORY_ALLOCATE_INFO, &flags, size, memory_type_index,
    };
    r = vkAllocateMemory(device, &mai, NULL, memory);
    if (r != VK_SUCCESS) {
        vkDestroyBuffer(device, *buffer, NULL);
        *buffer = VK_NULL_HANDLE;
        return r;
    }
    r = vkBindBufferMemory(device, *buffer, *memory, 0);
    if (r != VK_SUCCESS) {
        vkFreeMemory(device, *memory, NULL);
        vkDestroyBuffer(device, *buffer, NULL);
        *buffer = VK_NULL_HANDLE;
        *memory = VK_NULL_HANDLE;
    }
    return r;
}

/* One StateSet's draws from the imported command and count buffers: the
 * pass wrote counts[s] commands of 20 bytes (VkDrawIndexedIndirectCommand)
 * from command offsets[s] (the cadr_cull output layout). */
void cadr_vk_draw_state_set(VkCommandBuffer cb, VkBuffer cmds, VkBuffer counts, uint32_t state_set,
                            uint32_t region_start, uint32_t region_size)
{
    vkCmdDrawIndexedIndirectCount(cb, cmds, (VkDeviceSize)region_start * sizeof(VkDrawIndexedIndirectCommand),
                                  counts, (VkDeviceSize)state_set * sizeof(uint32_t), region_size,
                                  sizeof(VkDrawIndexedIndirectCommand));
}
