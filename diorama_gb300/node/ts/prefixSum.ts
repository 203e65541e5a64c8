// PrefixSum (src/prefixSum.ts:10-103) over the addon: an exclusive scan of u32
// values in place, `total` holding the sum. Untested: node is absent here.
import { native, NativeBuffer, NativeDevice } from './native';

export class PrefixSum {
  readonly total: NativeBuffer;
  private readonly handle: unknown;

  constructor(device: NativeDevice, data: NativeBuffer, capacity: number, count?: NativeBuffer) {
    this.handle = native.prefixSumCreate(device.handle, data.handle, capacity, count?.handle);
    this.total = new NativeBuffer(native.prefixSumTotal(this.handle));
  }

  // The pass argument of the WebGPU version is not needed: work is enqueued at once.
  encode(_pass?: unknown): void {
    native.prefixSumEncode(this.handle);
  }

  destroy(): void {
    native.prefixSumDestroy(this.handle);
  }
}
