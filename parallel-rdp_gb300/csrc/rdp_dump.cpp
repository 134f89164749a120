/*
 * RDPDUMP2 capture files: writer and replayer.
 *
 * The file format is the reference's (parallel-rdp/rdp_dump_write.cpp, rdp_dump.cpp): the
 * 8-byte tag "RDPDUMP2", the RDRAM and hidden-RDRAM sizes as 32-bit words, then records that
 * each start with a 32-bit command: 1 RDRAM block (offset, size, bytes), 2 RDP command (op,
 * word count, words), 3 VI register (index, value), 4 end of frame, 5 signal complete, 6 end of
 * file, 7 apply the RDRAM blocks so far, 8 hidden-RDRAM block, 9 apply the hidden blocks.  The
 * writer emits only the 4 KiB blocks that changed since the last flush, as the reference does.
 *
 * The replayer drives a processor the way the reference's replayer drives its
 * CommandProcessor (replayer_driver_parallel.cpp): block flushes become end_write_rdram /
 * end_write_hidden_rdram after the processor is idle, commands are enqueued, end of frame runs
 * a scanout (previous-frame blend on, no upscale de-interlacing) and hands the image to a
 * callback, signal complete flushes.
 */
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <new>
#include <vector>

#include "../../include/rdp_cuda.h"

struct rdp_dump_writer
{
	FILE *file = nullptr;
	std::vector<uint8_t> dram_cache, hidden_cache;

	void word(uint32_t v) { fwrite(&v, sizeof(v), 1, file); }

	void flush(const uint8_t *data, uint32_t size, std::vector<uint8_t> &cache, uint32_t block_cmd, uint32_t flush_cmd)
	{
		const uint32_t block = 4096;
		size = std::min<uint32_t>(size, uint32_t(cache.size()));
		for (uint32_t i = 0; i < size; i += block)
		{
			uint32_t n = std::min(block, size - i);
			if (memcmp(data + i, cache.data() + i, n) != 0)
			{
				word(block_cmd);
				word(i);
				word(n);
				fwrite(data + i, 1, n, file);
				memcpy(cache.data() + i, data + i, n);
			}
		}
		word(flush_cmd);
	}
};

namespace {
enum : uint32_t
{
	DUMP_UPDATE_DRAM = 1,
	DUMP_RDP_COMMAND = 2,
	DUMP_SET_VI_REGISTER = 3,
	DUMP_END_FRAME = 4,
	DUMP_SIGNAL_COMPLETE = 5,
	DUMP_EOF = 6,
	DUMP_UPDATE_DRAM_FLUSH = 7,
	DUMP_UPDATE_HIDDEN_DRAM = 8,
	DUMP_UPDATE_HIDDEN_DRAM_FLUSH = 9
};

bool read_u32(FILE *f, uint32_t &v) { return fread(&v, sizeof(v), 1, f) == 1; }
} // namespace

extern "C" {

int rdp_dump_writer_open(const char *path, uint32_t rdram_size, uint32_t hidden_rdram_size, rdp_dump_writer **out)
{
	if (!path || !out || !rdram_size || !hidden_rdram_size) return RDP_ERR_INVALID;
	*out = nullptr;
	rdp_dump_writer *w = new (std::nothrow) rdp_dump_writer();
	if (!w) return RDP_ERR_OOM;
	w->file = fopen(path, "wb");
	if (!w->file)
	{
		delete w;
		return RDP_ERR_INVALID;
	}
	w->dram_cache.assign(rdram_size, 0);
	w->hidden_cache.assign(hidden_rdram_size, 0);
	fwrite("RDPDUMP2", 8, 1, w->file);
	w->word(rdram_size);
	w->word(hidden_rdram_size);
	*out = w;
	return RDP_OK;
}

int rdp_dump_writer_flush_rdram(rdp_dump_writer *w, const void *rdram, uint32_t size)
{
	if (!w || !rdram) return RDP_ERR_INVALID;
	w->flush(static_cast<const uint8_t *>(rdram), size, w->dram_cache, DUMP_UPDATE_DRAM, DUMP_UPDATE_DRAM_FLUSH);
	return RDP_OK;
}

int rdp_dump_writer_flush_hidden_rdram(rdp_dump_writer *w, const void *hidden, uint32_t size)
{
	if (!w || !hidden) return RDP_ERR_INVALID;
	w->flush(static_cast<const uint8_t *>(hidden), size, w->hidden_cache, DUMP_UPDATE_HIDDEN_DRAM,
	         DUMP_UPDATE_HIDDEN_DRAM_FLUSH);
	return RDP_OK;
}

int rdp_dump_writer_command(rdp_dump_writer *w, uint32_t op, const uint32_t *words, uint32_t num_words)
{
	if (!w || (num_words && !words)) return RDP_ERR_INVALID;
	w->word(DUMP_RDP_COMMAND);
	w->word(op);
	w->word(num_words);
	if (num_words) fwrite(words, sizeof(uint32_t), num_words, w->file);
	return RDP_OK;
}

int rdp_dump_writer_set_vi_register(rdp_dump_writer *w, uint32_t reg, uint32_t value)
{
	if (!w) return RDP_ERR_INVALID;
	w->word(DUMP_SET_VI_REGISTER);
	w->word(reg);
	w->word(value);
	return RDP_OK;
}

int rdp_dump_writer_end_frame(rdp_dump_writer *w)
{
	if (!w) return RDP_ERR_INVALID;
	w->word(DUMP_END_FRAME);
	return RDP_OK;
}

int rdp_dump_writer_signal_complete(rdp_dump_writer *w)
{
	if (!w) return RDP_ERR_INVALID;
	w->word(DUMP_SIGNAL_COMPLETE);
	return RDP_OK;
}

int rdp_dump_writer_close(rdp_dump_writer *w)
{
	if (!w) return RDP_ERR_INVALID;
	w->word(DUMP_EOF);
	int r = fclose(w->file) == 0 ? RDP_OK : RDP_ERR_INVALID;
	delete w;
	return r;
}

int rdp_dump_replay(rdp_cp *cp, const char *path, rdp_dump_frame_cb on_frame, void *user, uint32_t *frames_out)
{
	if (!cp || !path) return RDP_ERR_INVALID;
	if (frames_out) *frames_out = 0;
	FILE *f = fopen(path, "rb");
	if (!f) return RDP_ERR_INVALID;
	char tag[8];
	uint32_t dram_size = 0, hidden_size = 0;
	int r = RDP_OK;
	if (fread(tag, 1, 8, f) != 8 || memcmp(tag, "RDPDUMP2", 8) != 0 || !read_u32(f, dram_size) ||
	    !read_u32(f, hidden_size) || dram_size > rdp_cp_get_rdram_size(cp) || hidden_size > rdp_cp_get_hidden_rdram_size(cp))
	{
		fclose(f);
		return RDP_ERR_INVALID;
	}
	std::vector<uint8_t> dram(dram_size, 0), hidden(hidden_size, 0);
	std::vector<uint32_t> cmd;
	std::vector<uint32_t> image(640 * 576);
	uint32_t frames = 0;
	rdp_scanout_options opts;
	rdp_scanout_options_default(&opts);
	opts.blend_previous_frame = 1;
	opts.upscale_deinterlacing = 0;
	for (bool done = false; !done && r == RDP_OK;)
	{
		uint32_t c;
		if (!read_u32(f, c))
		{
			r = RDP_ERR_INVALID;
			break;
		}
		switch (c)
		{
		case DUMP_EOF:
			done = true;
			break;
		case DUMP_SET_VI_REGISTER:
		{
			uint32_t idx, v;
			if (!read_u32(f, idx) || !read_u32(f, v)) r = RDP_ERR_INVALID;
			else r = rdp_cp_set_vi_register(cp, idx, v);
			break;
		}
		case DUMP_RDP_COMMAND:
		{
			uint32_t op, n;
			if (!read_u32(f, op) || !read_u32(f, n) || n > (1u << 20))
			{
				r = RDP_ERR_INVALID;
				break;
			}
			cmd.resize(n);
			if (n && fread(cmd.data(), sizeof(uint32_t), n, f) != n) r = RDP_ERR_INVALID;
			else r = rdp_cp_enqueue(cp, n, cmd.data());
			break;
		}
		case DUMP_END_FRAME:
		{
			uint32_t w = 0, h = 0;
			r = rdp_cp_scanout_sync(cp, &opts, image.data(), &w, &h);
			if (r == RDP_OK && on_frame) on_frame(user, frames, image.data(), w, h);
			frames++;
			break;
		}
		case DUMP_SIGNAL_COMPLETE:
			r = rdp_cp_flush(cp);
			break;
		case DUMP_UPDATE_DRAM:
		case DUMP_UPDATE_HIDDEN_DRAM:
		{
			uint32_t off, n;
			std::vector<uint8_t> &dst = c == DUMP_UPDATE_DRAM ? dram : hidden;
			if (!read_u32(f, off) || !read_u32(f, n) || uint64_t(off) + n > dst.size() ||
			    fread(dst.data() + off, 1, n, f) != n)
				r = RDP_ERR_INVALID;
			break;
		}
		case DUMP_UPDATE_DRAM_FLUSH:
		{
			uint8_t *p = static_cast<uint8_t *>(rdp_cp_begin_read_rdram(cp)); // idles the processor
			if (!p)
			{
				r = RDP_ERR_DEVICE;
				break;
			}
			memcpy(p, dram.data(), dram.size());
			r = rdp_cp_end_write_rdram(cp);
			break;
		}
		case DUMP_UPDATE_HIDDEN_DRAM_FLUSH:
		{
			uint8_t *p = static_cast<uint8_t *>(rdp_cp_begin_read_hidden_rdram(cp));
			if (!p)
			{
				r = RDP_ERR_DEVICE;
				break;
			}
			memcpy(p, hidden.data(), hidden.size());
			r = rdp_cp_end_write_hidden_rdram(cp);
			break;
		}
		default:
			r = RDP_ERR_INVALID;
			break;
		}
	}
	fclose(f);
	if (frames_out) *frames_out = frames;
	if (r == RDP_OK) r = rdp_cp_idle(cp);
	return r;
}

} // extern "C"
