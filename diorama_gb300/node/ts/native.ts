// The addon (diorama.node, built from ../diorama.cc) and the two objects the
// reference's classes take from WebGPU: the device (here a library context: one
// GPU and one in-order stream) and buffers (opaque handles). Untested: node is
// not installed on the machines this library was built on.
// eslint-disable-next-line @typescript-eslint/no-var-requires
export const native = require('../build/Release/diorama.node');

export type Handle = unknown;

export class NativeDevice {
  readonly handle: Handle;
  constructor(index = 0) {
    this.handle = native.contextCreate(index);
  }
  createBuffer(size: number): NativeBuffer {
    return new NativeBuffer(native.bufferCreate(this.handle, size), true);
  }
  // queue.writeBuffer: the data is copied at call time.
  writeBuffer(buffer: NativeBuffer, offset: number, data: ArrayBufferView): void {
    native.bufferWrite(buffer.handle, offset, data);
  }
  destroy(): void {
    native.contextDestroy(this.handle);
  }
}

export class NativeBuffer {
  constructor(
    readonly handle: Handle,
    private readonly owned = false,
  ) {}
  // readBuffer (src/readback.ts): resolves once the queued work before it is done.
  read(): Promise<ArrayBuffer> {
    return native.bufferRead(this.handle);
  }
  destroy(): void {
    if (this.owned) native.bufferDestroy(this.handle);
  }
}
