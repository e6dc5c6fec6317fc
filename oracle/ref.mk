# Builds the reference renderer's CPU path from its own C sources, where they lie, into
# oracle/_ref/libartref.so, together with oracle/refHarness.c.  Test infrastructure only: it pins the
# oracle restatement and generates the golden fixtures.  It needs the reference checkout (REF) and an
# x86-64 or aarch64 gcc; the reference's own CMake build is not used.
#
#   make -f oracle/ref.mk REF=/path/to/artful -j8
ifeq ($(REF),)
  $(error REF must name the reference checkout)
endif
HERE := $(dir $(lastword $(MAKEFILE_LIST)))
OUT := $(HERE)_ref
CC ?= gcc

# The reference's library sources minus the Vulkan and Metal backends (CMakeLists.txt:37-41).
SRCS := core/base.c core/threads.c \
  scene/scene.c scene/blocks.c scene/meshBuild.c scene/simplify.c scene/hole.c scene/fluid.c scene/trace.c \
  scene/gltf.c scene/imageDecode.c scene/graph.c scene/texture.c scene/environment.c scene/extras.c scene/meshopt.c \
  render/renderer.c \
  software/software.c software/post.c software/shadows.c software/denoise.c software/kernelsPortable.c

# The reference's own flags (CMakeLists.txt:55-57): no contraction, so every ISA draws the same bits.
CFLAGS := -std=c11 -O3 -fPIC -ffp-contract=off -fno-math-errno -fno-trapping-math -w \
  -I$(REF)/include -I$(REF)/src -D_GNU_SOURCE

ARCH := $(shell uname -m)
ifeq ($(ARCH),x86_64)
  SRCS += software/kernelsAvx2.c software/kernelsSse41.c
  CFLAGS += -DARTFUL_HAVE_AVX2 -DARTFUL_HAVE_SSE41
  FLAGS_kernelsAvx2 := -mavx2 -mno-fma
  FLAGS_kernelsSse41 := -msse4.1
else
  SRCS += software/kernelsNeon.c
  CFLAGS += -DARTFUL_HAVE_NEON
endif

OBJS := $(patsubst %.c,$(OUT)/obj/%.o,$(SRCS)) $(OUT)/obj/refHarness.o

$(OUT)/libartref.so: $(OBJS)
	$(CC) -shared -o $@ $^ -lm -lpthread

$(OUT)/obj/%.o: $(REF)/src/%.c
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) $(FLAGS_$(basename $(notdir $<))) -c $< -o $@

$(OUT)/obj/refHarness.o: $(HERE)refHarness.c
	@mkdir -p $(dir $@)
	$(CC) $(CFLAGS) -c $< -o $@

.PHONY: clean
clean:
	rm -rf $(OUT)
