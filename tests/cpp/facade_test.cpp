// Drives librdp_cuda through the header-only RDP::CommandProcessor facade (include/rdp_cuda.hpp) the
// way an emulator written against the reference's class does.  Used by tests/test_facade_gpu.py,
// which compares what this program writes with the oracle.
//
//   facade_test <words.bin> <rdram.bin> <vi_regs.bin> <out_dir>
//
// words.bin: the frame's RDP command words; rdram.bin: the initial RDRAM (8 MiB); vi_regs.bin:
// (register, value) pairs of uint32.  Renders the frame twice:
//   sync      -- commands decoded on the calling thread, in uneven chunks (partial commands carried
//                over), signal_timeline / wait_for_timeline, then scanout_sync;
//   threaded  -- COMMAND_PROCESSOR_FLAG_COMMAND_THREAD_BIT: the same chunks through the command
//                ring, with the in-band meta ops MetaFlush and MetaSignalTimeline in the stream
//                (the timeline value handed out by signal_timeline, waited on while the thread
//                decodes), then scanout() (device image) and scanout_async_buffer().
// Writes <out_dir>/{sync,threaded}_rdram.bin and sync_vi.bin, threaded_vi_device.bin,
// threaded_vi_async.bin (width, height, then RGBA8 pixels), and checks the API contracts it can
// check by itself (exit code != 0 on failure).
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "rdp_cuda.hpp"

static std::vector<uint8_t> read_file(const char *path)
{
	std::vector<uint8_t> d;
	FILE *f = fopen(path, "rb");
	if (!f) return d;
	fseek(f, 0, SEEK_END);
	d.resize(size_t(ftell(f)));
	fseek(f, 0, SEEK_SET);
	if (fread(d.data(), 1, d.size(), f) != d.size()) d.clear();
	fclose(f);
	return d;
}

static bool write_file(const std::string &path, const void *data, size_t size)
{
	FILE *f = fopen(path.c_str(), "wb");
	if (!f) return false;
	bool ok = fwrite(data, 1, size, f) == size;
	fclose(f);
	return ok;
}

static bool write_image(const std::string &path, unsigned w, unsigned h, const uint32_t *px)
{
	std::vector<uint32_t> out(2 + size_t(w) * h);
	out[0] = w;
	out[1] = h;
	if (w && h) memcpy(out.data() + 2, px, size_t(w) * h * 4);
	return write_file(path, out.data(), out.size() * 4);
}

#define CHECK(x)                                                              \
	do                                                                        \
	{                                                                         \
		if (!(x))                                                             \
		{                                                                     \
			fprintf(stderr, "facade_test: check failed: %s (line %d)\n", #x, __LINE__); \
			return 1;                                                         \
		}                                                                     \
	} while (0)

struct Reports : RDP::ValidationInterface
{
	int count = 0;
	void report_rdp_crash(RDP::ValidationError, const char *) override { count++; }
};

// Command lengths in words (RDP ops), to cut chunks at command boundaries for the meta ops.
static unsigned cmd_words(uint32_t w0)
{
	switch ((w0 >> 24) & 63)
	{
	case 0x08: return 8;
	case 0x09: return 12;
	case 0x0a: return 24;
	case 0x0b: return 28;
	case 0x0c: return 24;
	case 0x0d: return 28;
	case 0x0e: return 40;
	case 0x0f: return 44;
	case 0x24:
	case 0x25: return 4;
	default: return 2;
	}
}

int main(int argc, char **argv)
{
	if (argc != 5) return 2;
	std::vector<uint8_t> wbytes = read_file(argv[1]), rdram0 = read_file(argv[2]), vib = read_file(argv[3]);
	const std::string out = argv[4];
	CHECK(!wbytes.empty() && rdram0.size() == (8u << 20));
	const uint32_t *words = reinterpret_cast<const uint32_t *>(wbytes.data());
	const size_t nwords = wbytes.size() / 4;
	const uint32_t *vi = reinterpret_cast<const uint32_t *>(vib.data());
	const size_t nvi = vib.size() / 8;
	RDP::ScanoutOptions opts;
	opts.blend_previous_frame = false;
	opts.upscale_deinterlacing = false;

	// --------------------------------------------------------------------- sync
	{
		std::vector<uint8_t> rdram(rdram0);
		RDP::CommandProcessor cp(0, rdram.data(), 0, rdram.size(), rdram.size() / 2, 0);
		CHECK(cp.device_is_supported());
		CHECK(cp.get_rdram_size() == rdram.size() && cp.get_hidden_rdram_size() == rdram.size() / 2);
		Reports reports;
		cp.set_validation_interface(&reports);
		RDP::Quirks q;
		cp.set_quirks(q);
		cp.begin_frame_context();
		for (size_t i = 0; i < nwords;)
		{
			size_t n = std::min<size_t>(nwords - i, 1 + (i * 7919) % 997); // uneven, cuts commands
			cp.enqueue_command(unsigned(n), words + i);
			i += n;
		}
		uint64_t v = cp.signal_timeline();
		CHECK(v == 1);
		cp.wait_for_timeline(v);
		CHECK(memcmp(cp.begin_read_rdram(), rdram.data(), rdram.size()) == 0); // the caller's buffer
		CHECK(write_file(out + "/sync_rdram.bin", rdram.data(), rdram.size()));
		CHECK(cp.get_tmem() != nullptr);
		for (size_t k = 0; k < nvi; k++) cp.set_vi_register(RDP::VIRegister(vi[2 * k]), vi[2 * k + 1]);
		std::vector<RDP::RGBA> colors;
		unsigned w = 0, h = 0;
		cp.scanout_sync(colors, w, h, opts);
		CHECK(w > 0 && h > 0 && colors.size() == size_t(w) * h);
		CHECK(write_image(out + "/sync_vi.bin", w, h, reinterpret_cast<const uint32_t *>(colors.data())));
	}

	// --------------------------------------------------------------------- command thread + meta ops
	{
		std::vector<uint8_t> rdram(rdram0);
		RDP::CommandProcessor cp(0, rdram.data(), 0, rdram.size(), rdram.size() / 2,
		                         RDP::COMMAND_PROCESSOR_FLAG_COMMAND_THREAD_BIT);
		CHECK(cp.device_is_supported());
		// Whole commands, a MetaFlush after every 1,000th, a MetaSignalTimeline halfway.
		size_t i = 0, cmds = 0;
		uint64_t half = 0;
		while (i < nwords)
		{
			unsigned n = cmd_words(words[i]);
			cp.enqueue_command(n, words + i);
			i += n;
			if (++cmds % 1000 == 0)
			{
				const uint32_t flush_op = 2u << 24;
				cp.enqueue_command(1, &flush_op);
			}
			if (!half && i >= nwords / 2) half = cp.signal_timeline();
		}
		CHECK(half == 1);
		cp.wait_for_timeline(half); // may run while the thread decodes the second half
		// An in-band MetaSignalTimeline with an explicit value, then the API's next value.
		const uint32_t sig[3] = { 1u << 24, 7u, 0u };
		cp.enqueue_command(3, sig);
		uint64_t last = cp.signal_timeline();
		CHECK(last == 2);
		cp.wait_for_timeline(last);
		cp.idle();
		const void *host = cp.begin_read_rdram();
		CHECK(host == rdram.data());
		CHECK(write_file(out + "/threaded_rdram.bin", rdram.data(), rdram.size()));
		for (size_t k = 0; k < nvi; k++) cp.set_vi_register(RDP::VIRegister(vi[2 * k]), vi[2 * k + 1]);
		RDP::ScanoutImage img = cp.scanout(opts);
		CHECK(img && img.width > 0 && img.height > 0);
		std::vector<uint32_t> px(size_t(img.width) * img.height);
		CHECK(cudaMemcpy(px.data(), img.pixels, px.size() * 4, cudaMemcpyDeviceToHost) == cudaSuccess);
		CHECK(write_image(out + "/threaded_vi_device.bin", img.width, img.height, px.data()));
		// The next frame's scanout (same registers) into an asynchronous host buffer.
		RDP::VIScanoutBuffer buffer;
		cp.scanout_async_buffer(buffer, opts);
		CHECK(buffer.width == img.width && buffer.height == img.height);
		buffer.fence.wait();
		CHECK(write_image(out + "/threaded_vi_async.bin", buffer.width, buffer.height, buffer.data()));
	}

	// --------------------------------------------------------------------- unsupported configuration
	{
		std::vector<uint8_t> rdram(1 << 20);
		// Super-sampled readback without an upscaling factor (Renderer::init_renderer refuses it).
		RDP::CommandProcessor cp(0, rdram.data(), 0, rdram.size(), rdram.size() / 2,
		                         RDP::COMMAND_PROCESSOR_FLAG_SUPER_SAMPLED_READ_BACK_BIT);
		CHECK(!cp.device_is_supported());
		cp.enqueue_command(1, words); // no effect, no crash
		CHECK(cp.signal_timeline() == 0 && cp.begin_read_rdram() == nullptr);
	}
	printf("facade_test ok\n");
	return 0;
}
